// capi_project.cu -- C ABI of the kernel combination and multigrid
// projection (project.cu): the drop-in subroutines inv_grid_iso_ /
// inv2fwd_iso_ and the combine / post-process entry points.  Host arrays in,
// host arrays out; one stream and grow-only scratch per host thread.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../include/surfatt_gb300.h"
#include "host_buf.cuh"
#include "project.cuh"

using namespace sgb;

namespace {

struct ProjCtx {
  bool init = false;
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int launches = 0;
  bool timed = false;
  DBuf adj, adjd, svs, svp, srho, vs, vp, ker, kd, scaled, gk, grad, cells, w, rng, absmax, upd,
      terms, tcells;
  ~ProjCtx() {
    if (!init) return;
    for (DBuf* d : {&adj, &adjd, &svs, &svp, &srho, &vs, &vp, &ker, &kd, &scaled, &gk, &grad,
                    &cells, &w, &rng, &absmax, &upd, &terms, &tcells})
      d->release();
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (st) cudaStreamDestroy(st);
  }
  int setup() {
    if (init) return SURFATT_OK;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ev0) != cudaSuccess || cudaEventCreate(&ev1) != cudaSuccess) {
      // a partial setup is undone, so that the next call starts afresh
      if (ev0) cudaEventDestroy(ev0);
      if (ev1) cudaEventDestroy(ev1);
      if (st) cudaStreamDestroy(st);
      ev0 = ev1 = nullptr;
      st = nullptr;
      cudaGetLastError();
      return SURFATT_CUDA_ERROR;
    }
    init = true;
    return SURFATT_OK;
  }
};

thread_local ProjCtx g_pc;

int h2d(ProjCtx& c, DBuf& b, const void* src, size_t bytes) {
  if (b.ensure(bytes)) return SURFATT_OOM;
  if (src && bytes) CK(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, c.st));
  return SURFATT_OK;
}

// Plan tables to the device.
int upload_plan(ProjCtx& c, const ProjPlan& plan, ProjTables* t, ProjDev* D) {
  proj_pack(plan, t);
  int r = h2d(c, c.cells, t->cells.data(), t->cells.size() * sizeof(int));
  r = r ? r : h2d(c, c.w, t->w.data(), t->w.size() * sizeof(double));
  r = r ? r : h2d(c, c.rng, t->rng.data(), t->rng.size() * sizeof(int2));
  if (r) return r;
  *D = proj_dev(plan, *t, c.cells.as<int>(), c.w.as<double>(), c.rng.as<int2>());
  return SURFATT_OK;
}

// src/eikon_solver_2d.f90:1607-1609 / :1684-1686: print and `stop`.
void locate_stop(const ProjPlan& P) {
  if (!host_exit_on_stop()) return;
  std::printf(" I cannot locate the receiver in the domain. %24.16E %24.16E %24.16E\n",
              P.bad_xyz[0], P.bad_xyz[1], P.bad_xyz[2]);
  std::fflush(stdout);
  std::exit(0);
}

int plan_or_stop(const double* xinv, const double* yinv, const double* zinv, int nxinv,
                 int nyinv, int nzinv, int nset, const double* vx, const double* vy,
                 const double* vz, int nx, int ny, int nz, int need, ProjPlan* plan,
                 bool stop) {
  if (!xinv || !yinv || !zinv || !vx || !vy || !vz) return SURFATT_BAD_ARG;
  const int r = proj_plan(xinv, yinv, zinv, nxinv, nyinv, nzinv, nset, vx, vy, vz, nx, ny, nz,
                          need, plan);
  if (r == 7) {
    if (stop) locate_stop(*plan);
    return SURFATT_BAD_ARG;
  }
  return r ? SURFATT_BAD_ARG : SURFATT_OK;
}

// combine_kernels + post_processing_for_kernel on the device, host arrays in
// and out; either part may be skipped (adj_s == NULL: ker / ker_density are
// inputs; xinv == NULL: no post-processing).
int kernel_gradient(int P, int nx, int ny, int nz, const double* adj_s, const double* adj_density,
                    const double* sen_vs, const double* sen_vp, const double* sen_rho,
                    const double* vs3d, const double* vp3d, int abr, int rho_scaling,
                    double kdensity_coe, const double* xinv, const double* yinv,
                    const double* zinv, int nxinv, int nyinv, int nzinv, int nset,
                    const double* xgrids, const double* ygrids, const double* zgrids,
                    double chi0, double weight, int nker, double* ker, double* ker_density,
                    double* gradient_s) {
  const bool combine = adj_s != nullptr, post = xinv != nullptr;
  if (nx < 2 || ny < 2 || nz < 2 || (combine && P < 1)) return SURFATT_BAD_ARG;
  if (combine && (!adj_density || !sen_vs || !sen_vp || !sen_rho || (!abr && (!vs3d || !vp3d))))
    return SURFATT_BAD_ARG;
  if (!combine && (!ker || (post && kdensity_coe > 0 && !ker_density))) return SURFATT_BAD_ARG;
  if (post && !gradient_s) return SURFATT_BAD_ARG;
  ProjPlan plan;
  if (post) {
    const int r = plan_or_stop(xinv, yinv, zinv, nxinv, nyinv, nzinv, nset, xgrids, ygrids,
                               zgrids, nx, ny, nz, 3, &plan, false);
    if (r) return r;
  }
  ProjCtx& c = g_pc;
  int r = c.setup();
  if (r) return r;
  const size_t N2 = (size_t)nx * ny, N3 = N2 * nz, NK = (size_t)nker * N3;
  const size_t d = sizeof(double);
  if (combine) {
    r = h2d(c, c.adj, adj_s, (size_t)P * N2 * d);
    r = r ? r : h2d(c, c.adjd, adj_density, (size_t)P * N2 * d);
    r = r ? r : h2d(c, c.svs, sen_vs, (size_t)P * N3 * d);
    r = r ? r : h2d(c, c.svp, sen_vp, (size_t)P * N3 * d);
    r = r ? r : h2d(c, c.srho, sen_rho, (size_t)P * N3 * d);
    r = r ? r : h2d(c, c.vs, abr ? nullptr : vs3d, N3 * d);
    r = r ? r : h2d(c, c.vp, abr ? nullptr : vp3d, N3 * d);
    r = r ? r : h2d(c, c.ker, nullptr, NK * d);
    r = r ? r : h2d(c, c.kd, nullptr, NK * d);
  } else {
    r = h2d(c, c.ker, ker, NK * d);
    r = r ? r : h2d(c, c.kd, ker_density, (ker_density ? NK : 1) * d);
  }
  if (r) return r;
  ProjTables tabs;
  ProjDev D;
  if (post) {
    r = upload_plan(c, plan, &tabs, &D);
    const size_t ng = (size_t)nker * nset * nxinv * nyinv * nzinv;
    r = r ? r : h2d(c, c.grad, gradient_s, NK * d);
    r = r ? r : h2d(c, c.scaled, nullptr, NK * d);
    r = r ? r : h2d(c, c.gk, nullptr, ng * d);
    r = r ? r : h2d(c, c.absmax, nullptr, nker * sizeof(unsigned long long));
    r = r ? r : h2d(c, c.terms, nullptr, proj_terms_doubles(plan, nker) * d);
    r = r ? r : h2d(c, c.tcells, nullptr, proj_cells_ints(plan) * sizeof(int));
    if (r) return r;
  }
  CK(cudaEventRecord(c.ev0, c.st));
  c.launches = 0;
  if (combine) {
    launch_combine(P, nx, ny, nz, c.adj.as<double>(), c.adjd.as<double>(), c.svs.as<double>(),
                   c.svp.as<double>(), c.srho.as<double>(), c.vs.as<double>(), c.vp.as<double>(),
                   abr, rho_scaling, c.ker.as<double>(), c.kd.as<double>(), c.st);
    c.launches += 1;
  }
  if (post) {
    launch_post_process(D, nker, c.ker.as<double>(), c.kd.as<double>(), kdensity_coe,
                        c.scaled.as<double>(), c.terms.as<double>(), c.tcells.as<int>(),
                        c.gk.as<double>(), c.absmax.as<unsigned long long>(), chi0, weight,
                        c.grad.as<double>(), c.st);
    c.launches += kdensity_coe > 0 ? 5 : 4;
  }
  CK(cudaGetLastError());
  CK(cudaEventRecord(c.ev1, c.st));
  c.timed = true;
  if (ker) CK(cudaMemcpyAsync(ker, c.ker.p, NK * d, cudaMemcpyDeviceToHost, c.st));
  if (ker_density && combine)
    CK(cudaMemcpyAsync(ker_density, c.kd.p, NK * d, cudaMemcpyDeviceToHost, c.st));
  if (post) CK(cudaMemcpyAsync(gradient_s, c.grad.p, NK * d, cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  return SURFATT_OK;
}

}  // namespace

extern "C" {

void inv_grid_iso_(const double* xinv, const double* yinv, const double* zinv, const int* nxinv,
                   const int* nyinv, const int* nzinv, const int* nset, const double* adj,
                   const int* nx, const int* ny, const int* nz_3d, double* gk,
                   const double* vel_x, const double* vel_y, const double* vel_z_3d) {
  ProjPlan plan;
  int r = plan_or_stop(xinv, yinv, zinv, *nxinv, *nyinv, *nzinv, *nset, vel_x, vel_y, vel_z_3d,
                       *nx, *ny, *nz_3d, 1, &plan, true);
  if (r || !adj || !gk) {
    host_record(r ? r : SURFATT_BAD_ARG, 0);
    return;
  }
  ProjCtx& c = g_pc;
  if ((r = c.setup())) {
    host_record(r, 0);
    return;
  }
  const size_t N3 = (size_t)*nx * *ny * *nz_3d;
  const size_t ng = (size_t)*nset * *nxinv * *nyinv * *nzinv;
  ProjTables tabs;
  ProjDev D;
  r = upload_plan(c, plan, &tabs, &D);
  r = r ? r : h2d(c, c.ker, adj, N3 * sizeof(double));
  r = r ? r : h2d(c, c.scaled, nullptr, N3 * sizeof(double));
  r = r ? r : h2d(c, c.gk, nullptr, ng * sizeof(double));
  r = r ? r : h2d(c, c.terms, nullptr, proj_terms_doubles(plan, 1) * sizeof(double));
  r = r ? r : h2d(c, c.tcells, nullptr, proj_cells_ints(plan) * sizeof(int));
  if (!r) {
    launch_inv_grid(D, c.ker.as<double>(), c.scaled.as<double>(), c.terms.as<double>(),
                    c.tcells.as<int>(), c.gk.as<double>(), c.st);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(gk, c.gk.p, ng * sizeof(double), cudaMemcpyDeviceToHost, c.st) !=
            cudaSuccess ||
        cudaStreamSynchronize(c.st) != cudaSuccess)
      r = SURFATT_CUDA_ERROR;
  }
  host_record(r, 0);
}

void inv2fwd_iso_(const double* xinv, const double* yinv, const double* zinv, const int* nxinv,
                  const int* nyinv, const int* nzinv, const int* nset, const int* nx,
                  const int* ny, const int* nz_3d, const double* gk, const double* vel_x,
                  const double* vel_y, const double* vel_z_3d, double* update) {
  ProjPlan plan;
  int r = plan_or_stop(xinv, yinv, zinv, *nxinv, *nyinv, *nzinv, *nset, vel_x, vel_y, vel_z_3d,
                       *nx, *ny, *nz_3d, 2, &plan, true);
  if (r || !gk || !update) {
    host_record(r ? r : SURFATT_BAD_ARG, 0);
    return;
  }
  ProjCtx& c = g_pc;
  if ((r = c.setup())) {
    host_record(r, 0);
    return;
  }
  const size_t N3 = (size_t)*nx * *ny * *nz_3d;
  const size_t ng = (size_t)*nset * *nxinv * *nyinv * *nzinv;
  ProjTables tabs;
  ProjDev D;
  r = upload_plan(c, plan, &tabs, &D);
  r = r ? r : h2d(c, c.gk, gk, ng * sizeof(double));
  r = r ? r : h2d(c, c.upd, nullptr, N3 * sizeof(double));
  if (!r) {
    launch_inv2fwd(D, c.gk.as<double>(), c.upd.as<double>(), c.st);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(update, c.upd.p, N3 * sizeof(double), cudaMemcpyDeviceToHost, c.st) !=
            cudaSuccess ||
        cudaStreamSynchronize(c.st) != cudaSuccess)
      r = SURFATT_CUDA_ERROR;
  }
  host_record(r, 0);
}

surfatt_status_t surfatt_combine_kernels(int nperiod, int nx, int ny, int nz, const double* adj_s,
                                         const double* adj_density, const double* sen_vs,
                                         const double* sen_vp, const double* sen_rho,
                                         const double* vs3d, const double* vp3d,
                                         int use_alpha_beta_rho, int rho_scaling, double* ker,
                                         double* ker_density) {
  if (!adj_s || !ker || !ker_density) return SURFATT_BAD_ARG;
  return (surfatt_status_t)kernel_gradient(
      nperiod, nx, ny, nz, adj_s, adj_density, sen_vs, sen_vp, sen_rho, vs3d, vp3d,
      use_alpha_beta_rho, rho_scaling, 0.0, nullptr, nullptr, nullptr, 0, 0, 0, 0, nullptr,
      nullptr, nullptr, 1.0, 1.0, use_alpha_beta_rho ? 3 : 1, ker, ker_density, nullptr);
}

surfatt_status_t surfatt_post_process_kernels(int nker, int nx, int ny, int nz, double* ker,
                                              const double* ker_density, double kdensity_coe,
                                              const double* xinv, const double* yinv,
                                              const double* zinv, int nxinv, int nyinv,
                                              int nzinv, int nset, const double* xgrids,
                                              const double* ygrids, const double* zgrids,
                                              double chi0, double weight, double* gradient_s) {
  if (!xinv || nker < 1) return SURFATT_BAD_ARG;
  return (surfatt_status_t)kernel_gradient(
      0, nx, ny, nz, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0, 0,
      kdensity_coe, xinv, yinv, zinv, nxinv, nyinv, nzinv, nset, xgrids, ygrids, zgrids, chi0,
      weight, nker, ker, const_cast<double*>(ker_density), gradient_s);
}

surfatt_status_t surfatt_kernel_gradient(
    int nperiod, int nx, int ny, int nz, const double* adj_s, const double* adj_density,
    const double* sen_vs, const double* sen_vp, const double* sen_rho, const double* vs3d,
    const double* vp3d, int use_alpha_beta_rho, int rho_scaling, double kdensity_coe,
    const double* xinv, const double* yinv, const double* zinv, int nxinv, int nyinv, int nzinv,
    int nset, const double* xgrids, const double* ygrids, const double* zgrids, double chi0,
    double weight, double* ker, double* ker_density, double* gradient_s) {
  if (!adj_s || !xinv) return SURFATT_BAD_ARG;
  return (surfatt_status_t)kernel_gradient(
      nperiod, nx, ny, nz, adj_s, adj_density, sen_vs, sen_vp, sen_rho, vs3d, vp3d,
      use_alpha_beta_rho, rho_scaling, kdensity_coe, xinv, yinv, zinv, nxinv, nyinv, nzinv,
      nset, xgrids, ygrids, zgrids, chi0, weight, use_alpha_beta_rho ? 3 : 1, ker, ker_density,
      gradient_s);
}

surfatt_status_t surfatt_kernel_gradient_timing(double* kernel_ms, int* launches) {
  ProjCtx& c = g_pc;
  if (!c.timed) return SURFATT_BAD_ARG;
  CK(cudaEventSynchronize(c.ev1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
  if (kernel_ms) *kernel_ms = ms;
  if (launches) *launches = c.launches;
  return SURFATT_OK;
}

}  // extern "C"
