// capi.cu -- host side of libsurfatt_gb300.so: the drop-in Fortran symbols,
// the att_measadj mirror and the batched gradient-evaluation engine.
//
// There is no CPU path here: every solve runs on the GPU, and a missing or
// failing device is reported as SURFATT_CUDA_ERROR.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <numeric>
#include <vector>

#include "../../include/surfatt_gb300.h"
#include "host_buf.cuh"
#include "kernels.cuh"
#include "launch.cuh"
#include "smooth.cuh"

using namespace sgb;

namespace {

thread_local int g_last_status = SURFATT_OK;
thread_local int g_last_iters = 0;
int g_exit_on_boundary = 1;

// ---------------------------------------------------------------------------
// Per-thread drop-in context: one stream and grow-only scratch per host
// thread (the reference runs one solver per MPI rank; several ranks or
// threads may share a GPU).
// ---------------------------------------------------------------------------
struct PeriodBufs {
  DBuf xdeg, ydeg, xs, ys, cosy, siny, a, b, c, fun, f2, disx, disy, A, B, C, V;
  int ensure(int nx, int ny) {
    const size_t N = (size_t)nx * ny * sizeof(double);
    const size_t X = nx * sizeof(double), Y = ny * sizeof(double);
    int e = 0;
    e |= xdeg.ensure(X) | ydeg.ensure(Y) | xs.ensure(X) | ys.ensure(Y) | cosy.ensure(Y) |
         siny.ensure(Y);
    e |= a.ensure(N) | b.ensure(N) | c.ensure(N) | fun.ensure(N) | f2.ensure(N) |
         disx.ensure(N) | disy.ensure(N) | A.ensure(N) | B.ensure(N) | C.ensure(N) |
         V.ensure(N);
    return e ? SURFATT_OOM : SURFATT_OK;
  }
  void release() {
    for (DBuf* d : {&xdeg, &ydeg, &xs, &ys, &cosy, &siny, &a, &b, &c, &fun, &f2, &disx, &disy,
                    &A, &B, &C, &V})
      d->release();
  }
  PrepOut out() {
    return PrepOut{xs.as<double>(), ys.as<double>(), cosy.as<double>(), siny.as<double>(),
                   a.as<double>(), b.as<double>(), c.as<double>(), fun.as<double>(),
                   f2.as<double>(), disx.as<double>(), disy.as<double>(), nullptr, nullptr,
                   nullptr, nullptr};
  }
  PeriodDev dev(int nx, int ny, int lonlat, double dx, double dy, const double* svel) {
    PeriodDev P;
    P.nx = nx;
    P.ny = ny;
    P.lonlat = lonlat;
    P.dx = dx;
    P.dy = dy;
    P.xs = xs.as<double>();
    P.ys = ys.as<double>();
    P.xdeg = xdeg.as<double>();
    P.ydeg = ydeg.as<double>();
    P.cosy = cosy.as<double>();
    P.siny = siny.as<double>();
    P.a = a.as<double>();
    P.b = b.as<double>();
    P.c = c.as<double>();
    P.fun = fun.as<double>();
    P.f2 = f2.as<double>();
    P.disx = disx.as<double>();
    P.disy = disy.as<double>();
    P.svel = svel;
    P.goff = 0;
    P.f32 = nullptr;
    P.isv = nullptr;
    P.p4a = nullptr;
    P.p4b = nullptr;
    return P;
  }
};

struct ThreadCtx {
  bool init = false;
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;  // blocking-sync event: the end of a call's work
  PeriodBufs pb;
  DBuf ws, T, Ta, rx, ry, sa, out, si;
  DBuf sm_lon, sm_lat, sm_in, sm_out, sm_tab, sm_nyw, sm_per;  // kernel smoothing
  SmoothPlan sm_plan;            // plan of the table on the device
  std::vector<double> sm_key;    // nx, ny, sigma, lons, lats of that table
  int* si_host = nullptr;  // pinned {status, iters}
  // Pinned staging for the host <-> device copies of a call.  The caller's
  // arrays are pageable (Fortran arrays); a copy from pageable memory goes
  // through the driver's own staging buffer, which the threads of a process
  // share and take turns on.  Each call copies through its own thread's
  // pinned buffer instead (sized per call, offsets bumped per copy, reused
  // after the call's final synchronisation).
  double* hst = nullptr;
  size_t hst_cap = 0, hst_off = 0;
  // What the device already holds, as host copies of the inputs it came
  // from (compared bit for bit at the next call): consecutive calls of a
  // rank share the grid, metric and slowness, the adjoint takes the travel
  // times the forward call just returned, and the mask the adjoint field
  // the adjoint call just returned.  A matching input is not sent again.
  bool grid_ok = false, v_ok = false, v_null = false, t_ok = false, out_ok = false;
  int gk_nx = -1, gk_ny = -1, gk_flags = -1;
  std::vector<double> gk;  // xx | yy | A | B | C of the grid on the device
  std::vector<double> vk;  // its V (slowness or velocity)
  std::vector<double> tk;  // content of T (device)
  std::vector<double> ok;  // content of out (device)
  ~ThreadCtx() {
    if (!init) return;
    pb.release();
    for (DBuf* d : {&ws, &T, &Ta, &rx, &ry, &sa, &out, &si, &sm_lon, &sm_lat, &sm_in, &sm_out,
                    &sm_tab, &sm_nyw, &sm_per})
      d->release();
    if (si_host) cudaFreeHost(si_host);
    if (hst) cudaFreeHost(hst);
    if (done) cudaEventDestroy(done);
    if (st) cudaStreamDestroy(st);
  }
  int setup() {
    if (init) return SURFATT_OK;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
        cudaMallocHost(&si_host, 4 * sizeof(int)) == cudaSuccess &&
        cudaEventCreateWithFlags(&done, cudaEventBlockingSync | cudaEventDisableTiming) ==
            cudaSuccess) {
      init = true;
      return SURFATT_OK;
    }
    // a partial setup is undone, so that the next call starts afresh
    if (done) cudaEventDestroy(done);
    if (si_host) cudaFreeHost(si_host);
    if (st) cudaStreamDestroy(st);
    done = nullptr;
    si_host = nullptr;
    st = nullptr;
    cudaGetLastError();
    return SURFATT_CUDA_ERROR;
  }
  // Waits for the thread's stream, the calling thread sleeping rather than
  // spinning: callers on every host core (the reference's one MPI rank per
  // core) would otherwise keep each other's finished calls off the cores.
  cudaError_t wait() {
    const cudaError_t e = cudaEventRecord(done, st);
    return e != cudaSuccess ? e : cudaEventSynchronize(done);
  }
  // start of a call: room for `doubles` staged doubles
  int stage_begin(size_t doubles) {
    hst_off = 0;
    if (doubles <= hst_cap) return SURFATT_OK;
    if (hst) cudaFreeHost(hst);
    hst = nullptr;
    hst_cap = 0;
    if (cudaMallocHost(&hst, doubles * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      return SURFATT_OOM;
    }
    hst_cap = doubles;
    return SURFATT_OK;
  }
  // n doubles of the staging buffer (filled from src when given)
  double* stage(const double* src, size_t n) {
    double* p = hst + hst_off;
    if (src && n) std::memcpy(p, src, n * sizeof(double));
    hst_off += (n + 1) & ~(size_t)1;  // 16-byte steps
    return p;
  }
};

thread_local ThreadCtx g_ctx;

int record(int st, int iters) {
  g_last_status = st;
  g_last_iters = iters;
  return st;
}

// Whether v[off, off + n) holds x[0, n) bit for bit.
bool same_as(const std::vector<double>& v, size_t off, const double* x, size_t n) {
  return v.size() >= off + n && (n == 0 || std::memcmp(v.data() + off, x, n * sizeof(double)) == 0);
}

// Host -> device through the thread's pinned staging.
int h2d(ThreadCtx& c, void* dev, const double* src, size_t n) {
  if (!n) return SURFATT_OK;
  double* p = c.stage(src, n);
  CK(cudaMemcpyAsync(dev, p, n * sizeof(double), cudaMemcpyHostToDevice, c.st));
  return SURFATT_OK;
}

// Staged doubles per call for an nx x ny grid and nr receivers.
size_t stage_doubles(int nx, int ny, int nr) {
  return 8 * (size_t)nx * ny + nx + ny + 3 * (size_t)(nr > 0 ? nr : 0) + 64;
}

// Upload one grid + fields and run the per-period precompute, unless the
// device already holds them.  need_v = false: the caller uses only the
// metric (the adjoint), so a grid whose metric matches is reused whatever
// slowness came with it.
int prep_single(ThreadCtx& c, const double* xx, const double* yy, int nx, int ny, const double* A,
                const double* B, const double* C, const double* V, int lonlat, int from_model,
                PeriodDev* P, bool need_v = true) {
  const size_t N = (size_t)nx * ny;
  const void* before = c.pb.A.p;
  if (c.pb.ensure(nx, ny)) return SURFATT_OOM;
  if (c.pb.A.p != before) c.grid_ok = c.v_ok = false;  // buffers moved
  const int flags = lonlat | (from_model << 1);
  const bool gsame = c.grid_ok && c.gk_nx == nx && c.gk_ny == ny && c.gk_flags == flags &&
                     same_as(c.gk, 0, xx, nx) && same_as(c.gk, nx, yy, ny) &&
                     same_as(c.gk, nx + ny, A, N) && same_as(c.gk, nx + ny + N, B, N) &&
                     same_as(c.gk, nx + ny + 2 * N, C, N);
  const bool vsame = gsame && c.v_ok && (V ? (!c.v_null && same_as(c.vk, 0, V, N)) : c.v_null);
  if (!gsame || (need_v && !vsame)) {
    if (!gsame) {
      c.grid_ok = c.v_ok = false;
      int e = h2d(c, c.pb.xdeg.p, xx, nx) | h2d(c, c.pb.ydeg.p, yy, ny) |
              h2d(c, c.pb.A.p, A, N) | h2d(c, c.pb.B.p, B, N) | h2d(c, c.pb.C.p, C, N);
      if (e) return SURFATT_CUDA_ERROR;
      c.gk.resize(nx + ny + 3 * N);
      std::memcpy(c.gk.data(), xx, nx * sizeof(double));
      std::memcpy(c.gk.data() + nx, yy, ny * sizeof(double));
      std::memcpy(c.gk.data() + nx + ny, A, N * sizeof(double));
      std::memcpy(c.gk.data() + nx + ny + N, B, N * sizeof(double));
      std::memcpy(c.gk.data() + nx + ny + 2 * N, C, N * sizeof(double));
      c.gk_nx = nx;
      c.gk_ny = ny;
      c.gk_flags = flags;
    }
    if (V) {
      if (h2d(c, c.pb.V.p, V, N)) return SURFATT_CUDA_ERROR;
      c.vk.assign(V, V + N);
    } else {
      CK(cudaMemsetAsync(c.pb.V.p, 0, N * sizeof(double), c.st));
      c.vk.clear();
    }
    c.v_null = V == nullptr;
    PrepIn in{nx, ny, lonlat, c.pb.xdeg.as<double>(), c.pb.ydeg.as<double>(), c.pb.A.as<double>(),
              c.pb.B.as<double>(), c.pb.C.as<double>(), c.pb.V.as<double>(), from_model};
    launch_prep(in, c.pb.out(), c.st);
    CK(cudaGetLastError());
    c.grid_ok = c.v_ok = true;
  }
  // dx, dy in sweep units: xx(2)-xx(1) after the same conversion as the device
  double dx, dy;
  if (lonlat) {
    dx = xx[1] / 180.0 * PI_S - xx[0] / 180.0 * PI_S;
    dy = yy[1] / 180.0 * PI_S - yy[0] / 180.0 * PI_S;
  } else {
    dx = xx[1] - xx[0];
    dy = yy[1] - yy[0];
  }
  *P = c.pb.dev(nx, ny, lonlat, dx, dy, nullptr);
  return SURFATT_OK;
}

// Status + iterations back (and n doubles of out_dev into staging, returned
// in *staged), then wait for the stream.
int finish_single(ThreadCtx& c, const DBuf& out_dev, size_t n, double** staged) {
  CK(cudaMemcpyAsync(c.si_host, c.si.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, c.st));
  if (staged) {
    *staged = c.stage(nullptr, n);
    CK(cudaMemcpyAsync(*staged, out_dev.p, n * sizeof(double), cudaMemcpyDeviceToHost, c.st));
  }
  CK(c.wait());
  return SURFATT_OK;
}

void boundary_stop(double x0, double y0) {
  if (!g_exit_on_boundary) return;
  // src/eikon_solver_2d.f90:863-867: print and `stop`
  std::printf(" source on the boundary, mesh error\n");
  std::printf(" %24.16E %24.16E\n", x0, y0);
  std::fflush(stdout);
  std::exit(0);
}

int uw_dropin(const double* xx, const double* yy, int nx, int ny, const double* A,
              const double* B, const double* C, double* T, const double* fun, double x0,
              double y0, int lonlat, int weno, int multi) {
  if (!xx || !yy || !A || !B || !C || !T || !fun || nx < (weno ? 4 : 2) || ny < (weno ? 4 : 2))
    return record(SURFATT_BAD_ARG, 0);
  ThreadCtx& c = g_ctx;
  int e = c.setup();
  if (!e) e = c.stage_begin(stage_doubles(nx, ny, 0));
  if (e) return record(e, 0);
  PeriodDev P;
  e = prep_single(c, xx, yy, nx, ny, A, B, C, fun, lonlat, 0, &P);
  if (e) return record(e, 0);
  const size_t N = (size_t)nx * ny;
  if (c.ws.ensure(single_ws_doubles(N) * sizeof(double)) || c.T.ensure(N * sizeof(double)) ||
      c.si.ensure(4 * sizeof(int)))
    return record(SURFATT_OOM, 0);
  const double xs0 = lonlat ? x0 / 180.0 * PI_S : x0;
  const double ys0 = lonlat ? y0 / 180.0 * PI_S : y0;
  c.t_ok = false;  // T is rewritten
  if (weno)
    launch_weno_single(P, xs0, ys0, multi, c.ws.as<double>(), c.T.as<double>(), c.si.as<int>(), c.st);
  else if (!launch_uw_cluster(P, xs0, ys0, c.ws.as<double>(), c.T.as<double>(), c.si.as<int>(),
                              c.st))
    launch_uw_single(P, xs0, ys0, c.ws.as<double>(), c.T.as<double>(), c.si.as<int>(), c.st);
  if (cudaGetLastError() != cudaSuccess) return record(SURFATT_CUDA_ERROR, 0);
  double* staged = nullptr;
  e = finish_single(c, c.T, N, &staged);
  if (e) return record(e, 0);
  const int st = c.si_host[0], it = c.si_host[1];
  if (st == SURFATT_SOURCE_ON_BOUNDARY) {
    boundary_stop(xs0, ys0);
    return record(st, 0);
  }
  if (st == SURFATT_OK || st == SURFATT_NOT_CONVERGED) {
    std::memcpy(T, staged, N * sizeof(double));
    c.tk.assign(staged, staged + N);
    c.t_ok = true;
  }
  return record(st, it);
}

int jse_dropin(const double* xx, const double* yy, int nx, int ny, const double* A,
               const double* B, const double* C, const double* T, double* Ta, const double* xr,
               const double* yr, const double* sadj, int nr, int lonlat) {
  if (!xx || !yy || !A || !B || !C || !T || !Ta || nx < 3 || ny < 3 || nr < 0 ||
      (nr > 0 && (!xr || !yr || !sadj)))
    return record(SURFATT_BAD_ARG, 0);
  ThreadCtx& c = g_ctx;
  int e = c.setup();
  if (!e) e = c.stage_begin(stage_doubles(nx, ny, nr));
  if (e) return record(e, 0);
  PeriodDev P;
  e = prep_single(c, xx, yy, nx, ny, A, B, C, nullptr, lonlat, 0, &P, false);
  if (e) return record(e, 0);
  const size_t N = (size_t)nx * ny;
  const size_t R = (size_t)(nr > 0 ? nr : 1) * sizeof(double);
  if (c.ws.ensure(single_ws_doubles(N) * sizeof(double)) || c.T.ensure(N * sizeof(double)) ||
      c.out.ensure(N * sizeof(double)) || c.rx.ensure(R) || c.ry.ensure(R) || c.sa.ensure(R) ||
      c.si.ensure(4 * sizeof(int)))
    return record(SURFATT_OOM, 0);
  if (!(c.t_ok && c.tk.size() == N && same_as(c.tk, 0, T, N))) {
    c.t_ok = false;
    if (h2d(c, c.T.p, T, N)) return record(SURFATT_CUDA_ERROR, 0);
    c.tk.assign(T, T + N);
    c.t_ok = true;
  }
  if (nr > 0 && (h2d(c, c.rx.p, xr, nr) || h2d(c, c.ry.p, yr, nr) || h2d(c, c.sa.p, sadj, nr)))
    return record(SURFATT_CUDA_ERROR, 0);
  c.out_ok = false;  // out is rewritten
  launch_jse_single(P, c.T.as<double>(), c.rx.as<double>(), c.ry.as<double>(), c.sa.as<double>(),
                    nr, c.ws.as<double>(), c.out.as<double>(), c.si.as<int>(), c.st);
  if (cudaGetLastError() != cudaSuccess) return record(SURFATT_CUDA_ERROR, 0);
  double* staged = nullptr;
  e = finish_single(c, c.out, N, &staged);
  if (e) return record(e, 0);
  const int st = c.si_host[0], it = c.si_host[1];
  if (st == SURFATT_OK || st == SURFATT_NOT_CONVERGED) {
    std::memcpy(Ta, staged, N * sizeof(double));
    c.ok.assign(staged, staged + N);
    c.out_ok = true;
  }
  return record(st, it);
}

int mask_dropin(const double* xx, const double* yy, int nx, int ny, double* tab, double x0,
                double y0) {
  if (!xx || !yy || !tab || nx < 2 || ny < 2) return record(SURFATT_BAD_ARG, 0);
  ThreadCtx& c = g_ctx;
  int e = c.setup();
  if (!e) e = c.stage_begin(stage_doubles(nx, ny, 0));
  if (e) return record(e, 0);
  const size_t N = (size_t)nx * ny;
  const void* before = c.pb.A.p;
  if (c.pb.ensure(nx, ny) || c.out.ensure(N * sizeof(double))) return record(SURFATT_OOM, 0);
  if (c.pb.A.p != before) c.grid_ok = c.v_ok = false;
  // the node coordinates: those of the grid on the device when they match
  if (!(c.grid_ok && c.gk_nx == nx && c.gk_ny == ny && same_as(c.gk, 0, xx, nx) &&
        same_as(c.gk, nx, yy, ny))) {
    c.grid_ok = c.v_ok = false;  // the device's axes change
    if (h2d(c, c.pb.xdeg.p, xx, nx) || h2d(c, c.pb.ydeg.p, yy, ny))
      return record(SURFATT_CUDA_ERROR, 0);
  }
  if (!(c.out_ok && c.ok.size() == N && same_as(c.ok, 0, tab, N))) {
    c.out_ok = false;
    if (h2d(c, c.out.p, tab, N)) return record(SURFATT_CUDA_ERROR, 0);
  }
  c.out_ok = false;
  PeriodDev P = c.pb.dev(nx, ny, 0, 0, 0, nullptr);
  launch_mask_single(P, c.out.as<double>(), x0, y0, c.st);
  double* staged = c.stage(nullptr, N);
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(staged, c.out.p, N * sizeof(double), cudaMemcpyDeviceToHost, c.st) ||
      c.wait())
    return record(SURFATT_CUDA_ERROR, 0);
  std::memcpy(tab, staged, N * sizeof(double));
  c.ok.assign(staged, staged + N);
  c.out_ok = true;
  return record(SURFATT_OK, 0);
}

}  // namespace

namespace sgb {
int host_record(int status, int iters) { return record(status, iters); }
bool host_exit_on_stop() { return g_exit_on_boundary != 0; }
}  // namespace sgb

// ===========================================================================
// 1. Drop-in symbols
// ===========================================================================
extern "C" {

void fsm_uw_ps_lonlat_2d_(const double* xx_deg, const double* yy_deg, const int* nx,
                          const int* ny, const double* spha, const double* sphb,
                          const double* sphc, double* T, const double* fun,
                          const double* x0_deg, const double* y0_deg, const double* /*u*/) {
  uw_dropin(xx_deg, yy_deg, *nx, *ny, spha, sphb, sphc, T, fun, *x0_deg, *y0_deg, 1, 0, 0);
}

void fsm_uw_ps_cart_2d_(const double* xx, const double* yy, const int* nx, const int* ny,
                        const double* a, const double* b, const double* c, double* T,
                        const double* fun, const double* x0, const double* y0,
                        const double* /*u*/) {
  uw_dropin(xx, yy, *nx, *ny, a, b, c, T, fun, *x0, *y0, 0, 0, 0);
}

void fsm_weno3_ps_2d_(const double* xx, const double* yy, const int* nx, const int* ny,
                      const double* a, const double* b, const double* c, double* T,
                      const double* fun, const double* x0, const double* y0, const double* /*u*/) {
  uw_dropin(xx, yy, *nx, *ny, a, b, c, T, fun, *x0, *y0, 0, 1, 0);
}

void fsm_weno3_ps_multi_2d_(const double* xx, const double* yy, const int* nx, const int* ny,
                            const double* a, const double* b, const double* c, double* T,
                            const double* fun, const double* x0, const double* y0,
                            const double* /*u*/) {
  uw_dropin(xx, yy, *nx, *ny, a, b, c, T, fun, *x0, *y0, 0, 1, 1);
}

void fsm_o1_jse_lonlat_2d_(const double* xx_deg, const double* yy_deg, const int* nx,
                           const int* ny, const double* spha, const double* sphb,
                           const double* sphc, const double* T, double* Ta,
                           const double* xrec_deg, const double* yrec_deg,
                           const double* sourceAdj, const int* nr) {
  jse_dropin(xx_deg, yy_deg, *nx, *ny, spha, sphb, sphc, T, Ta, xrec_deg, yrec_deg, sourceAdj,
             *nr, 1);
}

void fsm_o1_jse_2d_(const double* xx, const double* yy, const int* nx, const int* ny,
                    const double* a, const double* b, const double* c, const double* T,
                    double* Ta, const double* xrec, const double* yrec,
                    const double* sourceAdj, const int* nr) {
  jse_dropin(xx, yy, *nx, *ny, a, b, c, T, Ta, xrec, yrec, sourceAdj, *nr, 0);
}

void mask_(const double* xx, const double* yy, const int* nx, const int* ny, double* TableAdj,
           const double* x0, const double* y0) {
  mask_dropin(xx, yy, *nx, *ny, TableAdj, *x0, *y0);
}

int surfatt_last_status(void) { return g_last_status; }
int surfatt_last_iterations(void) { return g_last_iters; }
void surfatt_set_exit_on_boundary(int enable) { g_exit_on_boundary = enable; }
const char* surfatt_version(void) { return "surfatt_gb300 0.1 (sm_103a)"; }

// ===========================================================================
// 2. Measurement layer (src/measadj.f90)
// ===========================================================================
surfatt_status_t surfatt_measadj_run_forward(const double* xgrids, const double* ygrids,
                                             int nx, int ny, const double* vel2d,
                                             const double* m11, const double* m22,
                                             const double* m12, double srcx, double srcy,
                                             int nrec, const double* recx, const double* recy,
                                             const double* tt, const double* weight,
                                             double* timetable, double* tekio, double* chi) {
  if (!vel2d || !m11 || !m22 || !m12 || !timetable || nrec < 0 ||
      (nrec > 0 && (!recx || !recy || !tt || !weight || !tekio)) || !chi || nx < 2 || ny < 2)
    return (surfatt_status_t)record(SURFATT_BAD_ARG, 0);
  ThreadCtx& c = g_ctx;
  int e = c.setup();
  if (!e) e = c.stage_begin(stage_doubles(nx, ny, nrec));
  if (e) return (surfatt_status_t)record(e, 0);
  PeriodDev P;
  e = prep_single(c, xgrids, ygrids, nx, ny, m11, m22, m12, vel2d, 1, 1, &P);
  if (e) return (surfatt_status_t)record(e, 0);
  const size_t N = (size_t)nx * ny;
  const size_t R = (size_t)(nrec > 0 ? nrec : 1) * sizeof(double);
  if (c.ws.ensure(single_ws_doubles(N) * sizeof(double)) || c.T.ensure(N * sizeof(double)) ||
      c.si.ensure(4 * sizeof(int)) || c.rx.ensure(R) || c.ry.ensure(R) || c.sa.ensure(R))
    return (surfatt_status_t)record(SURFATT_OOM, 0);
  const double xs0 = srcx / 180.0 * PI_S, ys0 = srcy / 180.0 * PI_S;
  c.t_ok = false;  // T is rewritten
  if (!launch_uw_cluster(P, xs0, ys0, c.ws.as<double>(), c.T.as<double>(), c.si.as<int>(), c.st))
    launch_uw_single(P, xs0, ys0, c.ws.as<double>(), c.T.as<double>(), c.si.as<int>(), c.st);
  if (cudaMemsetAsync(c.si.as<int>() + 2, 0, sizeof(int), c.st) != cudaSuccess)
    return (surfatt_status_t)record(SURFATT_CUDA_ERROR, 0);
  if (nrec > 0) {
    if (h2d(c, c.rx.p, recx, nrec) || h2d(c, c.ry.p, recy, nrec))
      return (surfatt_status_t)record(SURFATT_CUDA_ERROR, 0);
    launch_interp(P, c.T.as<double>(), nrec, c.rx.as<double>(), c.ry.as<double>(),
                  c.sa.as<double>(), c.si.as<int>() + 2, c.st);
  }
  if (cudaGetLastError() != cudaSuccess) return (surfatt_status_t)record(SURFATT_CUDA_ERROR, 0);
  double* st_T = c.stage(nullptr, N);
  double* st_k = c.stage(nullptr, nrec > 0 ? nrec : 0);
  if (cudaMemcpyAsync(c.si_host, c.si.p, 3 * sizeof(int), cudaMemcpyDeviceToHost, c.st) ||
      cudaMemcpyAsync(st_T, c.T.p, N * sizeof(double), cudaMemcpyDeviceToHost, c.st) ||
      (nrec > 0 && cudaMemcpyAsync(st_k, c.sa.p, nrec * sizeof(double), cudaMemcpyDeviceToHost, c.st)) ||
      c.wait())
    return (surfatt_status_t)record(SURFATT_CUDA_ERROR, 0);
  std::memcpy(timetable, st_T, N * sizeof(double));
  if (nrec > 0) std::memcpy(tekio, st_k, nrec * sizeof(double));
  c.tk.assign(st_T, st_T + N);
  c.t_ok = true;
  int st = c.si_host[0];
  if (st == SURFATT_SOURCE_ON_BOUNDARY) return (surfatt_status_t)record(st, 0);
  if (nrec > 0 && c.si_host[2] != 0 && st == SURFATT_OK) st = SURFATT_BAD_ARG;
  // chi = 0.5*sum(weight*(tekio-tt)**2): a scalar of the receivers, summed in
  // receiver order on the host side of the call, as the reference does
  double s = 0;
  for (int i = 0; i < nrec; ++i) {
    const double d = tekio[i] - tt[i];
    s = s + weight[i] * (d * d);
  }
  *chi = 0.5 * s;
  return (surfatt_status_t)record(st, c.si_host[1]);
}

surfatt_status_t surfatt_measadj_run_adjoint(const double* xgrids, const double* ygrids,
                                             int nx, int ny, const double* m11,
                                             const double* m22, const double* m12,
                                             double srcx, double srcy, int nrec,
                                             const double* recx, const double* recy,
                                             const double* tt, const double* tekio,
                                             double* weight, const double* timetable,
                                             double* adjtable) {
  if (nrec < 0 || (nrec > 0 && (!tt || !tekio || !weight)) || !m12)
    return (surfatt_status_t)record(SURFATT_BAD_ARG, 0);
  std::vector<double> sadj((size_t)(nrec > 0 ? nrec : 1)), nm12((size_t)nx * ny);
  for (int i = 0; i < nrec; ++i)
    if (std::fabs(tekio[i] - tt[i]) / tt[i] > 0.5) weight[i] = 0.;
  for (int i = 0; i < nrec; ++i) sadj[i] = weight[i] * (tekio[i] - tt[i]);
  for (size_t k = 0; k < nm12.size(); ++k) nm12[k] = -m12[k];
  int st = jse_dropin(xgrids, ygrids, nx, ny, m11, m22, nm12.data(), timetable, adjtable, recx,
                      recy, sadj.data(), nrec, 1);
  if (st != SURFATT_OK && st != SURFATT_NOT_CONVERGED) return (surfatt_status_t)st;
  const int it = g_last_iters;
  int sm = mask_dropin(xgrids, ygrids, nx, ny, adjtable, srcx, srcy);
  if (sm != SURFATT_OK) return (surfatt_status_t)sm;
  return (surfatt_status_t)record(st, it);
}

surfatt_status_t surfatt_measadj_run_adjoint_density(
    const double* xgrids, const double* ygrids, int nx, int ny, const double* m11,
    const double* m22, const double* m12, double srcx, double srcy, int nrec,
    const double* recx, const double* recy, const double* weight, const double* timetable,
    double* density) {
  if (nrec < 0 || (nrec > 0 && !weight) || !m12) return (surfatt_status_t)record(SURFATT_BAD_ARG, 0);
  std::vector<double> sadj((size_t)(nrec > 0 ? nrec : 1)), nm12((size_t)nx * ny);
  for (int i = 0; i < nrec; ++i) sadj[i] = -1.0 * weight[i];
  for (size_t k = 0; k < nm12.size(); ++k) nm12[k] = -m12[k];
  int st = jse_dropin(xgrids, ygrids, nx, ny, m11, m22, nm12.data(), timetable, density, recx,
                      recy, sadj.data(), nrec, 1);
  if (st != SURFATT_OK && st != SURFATT_NOT_CONVERGED) return (surfatt_status_t)st;
  const int it = g_last_iters;
  int sm = mask_dropin(xgrids, ygrids, nx, ny, density, srcx, srcy);
  if (sm != SURFATT_OK) return (surfatt_status_t)sm;
  return (surfatt_status_t)record(st, it);
}

// gaussian_smooth_geo_2 (src/shared/utils.f90:1194-1225) of one (nx, ny) field.
surfatt_status_t surfatt_gaussian_smooth_geo_2(const double* data, int nx, int ny,
                                               const double* lons, const double* lats,
                                               double sigma, double* smdata) {
  if (!data || !lons || !lats || !smdata || nx < 2 || ny < 2)
    return (surfatt_status_t)record(SURFATT_BAD_ARG, 0);
  // The weight table depends on the grid and sigma only: a call with the
  // same ones as the previous call of this thread reuses it.
  std::vector<double> key((size_t)nx + ny + 3);
  key[0] = nx;
  key[1] = ny;
  key[2] = sigma;
  std::memcpy(key.data() + 3, lons, nx * sizeof(double));
  std::memcpy(key.data() + 3 + nx, lats, ny * sizeof(double));
  ThreadCtx& c = g_ctx;
  const bool cached = c.init && key.size() == c.sm_key.size() &&
                      std::memcmp(key.data(), c.sm_key.data(), key.size() * sizeof(double)) == 0;
  if (!cached) {
    SmoothPlan plan;
    const long long zero = 0;
    if (smooth_plan(1, &nx, &ny, &zero, nullptr, &zero, &zero, lons, lats, &sigma, &plan) !=
        ST_OK)
      return (surfatt_status_t)record(SURFATT_BAD_ARG, 0);
    int e = c.setup();
    if (e) return (surfatt_status_t)record(e, 0);
    c.sm_key.clear();
    if (c.sm_lon.ensure(nx * sizeof(double)) || c.sm_lat.ensure(ny * sizeof(double)) ||
        c.sm_tab.ensure((size_t)plan.table_doubles * sizeof(double)) ||
        c.sm_nyw.ensure((size_t)plan.nyw_count * sizeof(int)) ||
        c.sm_per.ensure(sizeof(SmoothPeriod)))
      return (surfatt_status_t)record(SURFATT_OOM, 0);
    c.sm_plan = plan;
  }
  const SmoothPlan& plan = c.sm_plan;
  const size_t N = (size_t)nx * ny;
  if (c.sm_in.ensure(N * sizeof(double)) || c.sm_out.ensure(N * sizeof(double)))
    return (surfatt_status_t)record(SURFATT_OOM, 0);
  CK(cudaMemcpyAsync(c.sm_in.p, data, N * sizeof(double), cudaMemcpyHostToDevice, c.st));
  SmoothArgs A{c.sm_per.as<SmoothPeriod>(), 1, c.sm_lon.as<double>(), c.sm_lat.as<double>(),
               c.sm_nyw.as<int>(), c.sm_in.as<double>(), c.sm_out.as<double>(),
               c.sm_tab.as<double>(), plan.nodes};
  if (!cached) {
    CK(cudaMemcpyAsync(c.sm_lon.p, lons, nx * sizeof(double), cudaMemcpyHostToDevice, c.st));
    CK(cudaMemcpyAsync(c.sm_lat.p, lats, ny * sizeof(double), cudaMemcpyHostToDevice, c.st));
    CK(cudaMemcpyAsync(c.sm_nyw.p, plan.nyw.data(), plan.nyw_count * sizeof(int),
                       cudaMemcpyHostToDevice, c.st));
    CK(cudaMemcpyAsync(c.sm_per.p, plan.per.data(), sizeof(SmoothPeriod),
                       cudaMemcpyHostToDevice, c.st));
    launch_smooth_table(A, plan, c.st);
    CK(cudaGetLastError());
  }
  launch_smooth_apply(A, plan, c.st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(smdata, c.sm_out.p, N * sizeof(double), cudaMemcpyDeviceToHost, c.st));
  CK(c.wait());
  c.sm_key.swap(key);
  return (surfatt_status_t)record(SURFATT_OK, 0);
}

}  // extern "C"

// ===========================================================================
// 3. Batched engine
// ===========================================================================
struct surfatt_engine {
  int device = 0;
  size_t budget = 0;
  size_t allocated = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evk0 = nullptr, evk1 = nullptr;
  bool loaded = false, ran = false;
  int last_mode = 0, launches = 0;
  // problem shape (host)
  int nperiod = 0, nsolve = 0, npath = 0, nrec_total = 0;
  long long ncell = 0, kslot_total = 0, max_cells = 0;
  std::vector<int> nx, ny, pidx, nrec;
  std::vector<long long> goff, xoff, yoff;
  std::vector<PeriodDev> periods;
  std::vector<int> order, plist_off, plist;
  std::vector<long long> kslot;
  // device buffers
  DBuf d_periods, d_xdeg, d_ydeg, d_xs, d_ys, d_cosy, d_siny, d_A, d_B, d_C, d_V, d_a, d_b, d_c,
      d_fun, d_f2, d_disx, d_disy, d_f32, d_isv, d_p4a, d_pidx, d_srcx, d_srcy, d_rec_off, d_nrec, d_recx, d_recy,
      d_tt, d_weight, d_path, d_order, d_plist_off, d_plist, d_kslot, d_goff, d_nx, d_ny;
  DBuf d_tekio, d_wgt, d_ttfwd, d_chis, d_chi, d_kc, d_kcd, d_adj, d_adjd, d_status, d_fit, d_ait,
      d_fupd, d_aupd, d_ws, d_queue, d_phase;
  // kernel smoothing of adj_s (gaussian_smooth_geo_2 per period)
  DBuf d_ker, d_smtab, d_smnyw, d_smper;
  std::vector<double> hx, hy;  // host copies of the grid axes (window plan)
  SmoothPlan smplan;
  double sm_sigma = -1.0;      // sigma of the weight table on the device (-1: none)
  bool smoothed = false;
  int sm_launches = 0;         // kernel launches of the last smoothing
  cudaEvent_t evs0 = nullptr, evs1 = nullptr;
  ClassStreams cs;  // side streams of the FP32 row kernel's team classes
  int grid = 0, block = 128, per_sm = 0, last_block = 0, last_kind = 0, last_pf = 0;
  size_t last_smem = 0;
  KernelChoice tuned[2];  // per precision; -1 fields: automatic
  // Captured evaluations: one executable graph per (mode, precision), valid
  // while the buffers and the problem shape it was captured on are unchanged
  // (`gen` moves on every load and every reallocation).
  struct Captured {
    cudaGraphExec_t exec = nullptr;
    long long gen = -1;
    int kind = -1, pf = -1, grid = 0, launches = 0;
  };
  Captured graphs[4][2];
  long long gen = 0;
  std::vector<long long> shape_sig;  // sizes of the loaded problem (see load)
  bool use_graphs = true;
  bool profile = false;  // per-phase cycle counters of the FP32 warp kernel
  bool keep_fields = false;  // write every solve's travel-time field (d_T)
  DBuf d_T;
  int hold_solve = -1, item_wait_limit = 0;  // test hooks of the bounded item wait
  void drop_graphs() {
    for (auto& m : graphs)
      for (auto& g : m) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = Captured();
      }
  }
  std::vector<DBuf*> all() {
    return {&d_periods, &d_xdeg, &d_ydeg, &d_xs, &d_ys, &d_cosy, &d_siny, &d_A, &d_B, &d_C,
            &d_V, &d_a, &d_b, &d_c, &d_fun, &d_f2, &d_disx, &d_disy, &d_f32, &d_isv, &d_p4a, &d_pidx, &d_srcx, &d_srcy,
            &d_rec_off, &d_nrec, &d_recx, &d_recy, &d_tt, &d_weight, &d_path, &d_order,
            &d_plist_off, &d_plist, &d_kslot, &d_goff, &d_nx, &d_ny, &d_tekio, &d_wgt, &d_ttfwd,
            &d_chis, &d_chi, &d_kc, &d_kcd, &d_adj, &d_adjd, &d_status, &d_fit, &d_ait, &d_fupd,
            &d_aupd, &d_ws, &d_queue, &d_phase, &d_ker, &d_smtab, &d_smnyw, &d_smper,
            &d_T};
  }
};

namespace {

int eng_ensure(surfatt_engine* e, DBuf& b, size_t bytes) {
  b.counter = &e->allocated;
  if (bytes <= b.cap) return SURFATT_OK;
  if (e->budget && e->allocated - b.cap + bytes > e->budget) return SURFATT_OOM;
  ++e->gen;  // a captured evaluation may hold the old pointer
  return b.ensure(bytes);
}

template <class T>
int up(surfatt_engine* e, DBuf& b, const T* src, size_t n) {
  int r = eng_ensure(e, b, (n ? n : 1) * sizeof(T));
  if (r) return r;
  if (n && src) CK(cudaMemcpyAsync(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice, e->st));
  return SURFATT_OK;
}

int run_prep_all(surfatt_engine* e) {
  std::vector<PrepIn> ins(e->nperiod);
  std::vector<PrepOut> outs(e->nperiod);
  for (int p = 0; p < e->nperiod; ++p) {
    const long long g = e->goff[p];
    ins[p] = PrepIn{e->nx[p], e->ny[p], 1, e->d_xdeg.as<double>() + e->xoff[p],
              e->d_ydeg.as<double>() + e->yoff[p], e->d_A.as<double>() + g,
              e->d_B.as<double>() + g, e->d_C.as<double>() + g, e->d_V.as<double>() + g, 1};
    outs[p] = PrepOut{e->d_xs.as<double>() + e->xoff[p], e->d_ys.as<double>() + e->yoff[p],
                e->d_cosy.as<double>() + e->yoff[p], e->d_siny.as<double>() + e->yoff[p],
                e->d_a.as<double>() + g, e->d_b.as<double>() + g, e->d_c.as<double>() + g,
                e->d_fun.as<double>() + g, e->d_f2.as<double>() + g,
                e->d_disx.as<double>() + g, e->d_disy.as<double>() + g,
                e->d_f32.as<float>() + 6 * g, e->d_isv.as<double>() + 2 * g,
                e->d_p4a.as<float4>() + 2 * g, e->d_p4a.as<float4>() + 2 * g + 1};
  }
  launch_prep_batch(ins.data(), outs.data(), e->nperiod, e->st);
  CK(cudaGetLastError());
  return SURFATT_OK;
}

}  // namespace

extern "C" {

surfatt_status_t surfatt_engine_create(surfatt_engine_t** out, int device, size_t budget) {
  if (!out) return SURFATT_BAD_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return SURFATT_CUDA_ERROR;
  }
  CK(cudaSetDevice(device));
  auto* e = new surfatt_engine();
  e->device = device;
  e->budget = budget;
  if (cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e->ev0) != cudaSuccess || cudaEventCreate(&e->ev1) != cudaSuccess ||
      cudaEventCreate(&e->evk0) != cudaSuccess || cudaEventCreate(&e->evk1) != cudaSuccess ||
      cudaEventCreate(&e->evs0) != cudaSuccess || cudaEventCreate(&e->evs1) != cudaSuccess ||
      e->cs.create() != ST_OK) {
    e->cs.destroy();
    for (cudaEvent_t ev : {e->ev0, e->ev1, e->evk0, e->evk1, e->evs0, e->evs1})
      if (ev) cudaEventDestroy(ev);
    if (e->st) cudaStreamDestroy(e->st);
    cudaGetLastError();
    delete e;
    return SURFATT_CUDA_ERROR;
  }
  *out = e;
  return SURFATT_OK;
}

void surfatt_engine_destroy(surfatt_engine_t* e) {
  if (!e) return;
  cudaSetDevice(e->device);
  cudaStreamSynchronize(e->st);
  e->drop_graphs();
  for (DBuf* b : e->all()) b->release();
  cudaEventDestroy(e->ev0);
  cudaEventDestroy(e->ev1);
  cudaEventDestroy(e->evk0);
  cudaEventDestroy(e->evk1);
  cudaEventDestroy(e->evs0);
  cudaEventDestroy(e->evs1);
  e->cs.destroy();
  cudaStreamDestroy(e->st);
  delete e;
}

surfatt_status_t surfatt_engine_load(surfatt_engine_t* e, const surfatt_problem_t* pb) {
  if (!e || !pb || pb->nperiod < 1 || pb->nsolve < 0) return SURFATT_BAD_ARG;
  CK(cudaSetDevice(e->device));
  e->loaded = false;
  e->ran = false;
  e->tuned[0] = e->tuned[1] = KernelChoice();
  const int np = pb->nperiod, ns = pb->nsolve;
  e->nperiod = np;
  e->nsolve = ns;
  e->npath = pb->npath;
  e->nx.assign(pb->nx, pb->nx + np);
  e->ny.assign(pb->ny, pb->ny + np);
  e->goff.assign(pb->goff, pb->goff + np);
  e->xoff.assign(pb->xoff, pb->xoff + np);
  e->yoff.assign(pb->yoff, pb->yoff + np);
  e->pidx.assign(pb->pidx, pb->pidx + ns);
  e->nrec.assign(pb->nrec, pb->nrec + ns);
  long long nxs = 0, nys = 0;
  e->ncell = 0;
  e->max_cells = 0;
  for (int p = 0; p < np; ++p) {
    if (e->nx[p] < 3 || e->ny[p] < 3) return SURFATT_BAD_ARG;
    const long long N = (long long)e->nx[p] * e->ny[p];
    e->ncell = std::max(e->ncell, e->goff[p] + N);
    e->max_cells = std::max(e->max_cells, N);
    nxs = std::max(nxs, e->xoff[p] + e->nx[p]);
    nys = std::max(nys, e->yoff[p] + e->ny[p]);
  }
  int nrec_total = 0;
  for (int s = 0; s < ns; ++s) {
    if (e->pidx[s] < 0 || e->pidx[s] >= np || e->nrec[s] < 0) return SURFATT_BAD_ARG;
    nrec_total = std::max(nrec_total, pb->rec_off[s] + e->nrec[s]);
  }
  for (int r = 0; r < nrec_total; ++r)
    if (pb->path[r] < 0 || pb->path[r] >= pb->npath) return SURFATT_BAD_ARG;
  e->nrec_total = nrec_total;
  // processing order: by team class of the FP32 row kernel (the class of
  // the tallest grids first, each class contiguous), then largest grids
  // first (longest-processing-time first)
  e->order.resize(ns);
  std::iota(e->order.begin(), e->order.end(), 0);
  std::stable_sort(e->order.begin(), e->order.end(), [&](int a, int b) {
    const int ka = team_class_key(e->ny[e->pidx[a]]), kb = team_class_key(e->ny[e->pidx[b]]);
    if (ka != kb) return ka > kb;
    return (long long)e->nx[e->pidx[a]] * e->ny[e->pidx[a]] >
           (long long)e->nx[e->pidx[b]] * e->ny[e->pidx[b]];
  });
  // per-period solve lists in work-list order, kernel slots per solve
  e->plist_off.assign(np + 1, 0);
  for (int s = 0; s < ns; ++s) e->plist_off[e->pidx[s] + 1]++;
  for (int p = 0; p < np; ++p) e->plist_off[p + 1] += e->plist_off[p];
  e->plist.assign(ns, 0);
  {
    std::vector<int> fill(e->plist_off.begin(), e->plist_off.end() - 1);
    for (int s = 0; s < ns; ++s) e->plist[fill[e->pidx[s]]++] = s;
  }
  e->kslot.assign(ns, 0);
  long long acc = 0;
  for (int s = 0; s < ns; ++s) {
    e->kslot[s] = acc;
    acc += (long long)e->nx[e->pidx[s]] * e->ny[e->pidx[s]];
  }
  e->kslot_total = acc;
  const size_t NC = (size_t)e->ncell;
  int r = 0;
  r |= up(e, e->d_xdeg, pb->xgrid, nxs) | up(e, e->d_ydeg, pb->ygrid, nys);
  e->hx.assign(pb->xgrid, pb->xgrid + nxs);
  e->hy.assign(pb->ygrid, pb->ygrid + nys);
  e->sm_sigma = -1.0;
  e->smoothed = false;
  r |= up(e, e->d_xs, (double*)nullptr, nxs) | up(e, e->d_ys, (double*)nullptr, nys);
  r |= up(e, e->d_cosy, (double*)nullptr, nys) | up(e, e->d_siny, (double*)nullptr, nys);
  r |= up(e, e->d_A, pb->m11, NC) | up(e, e->d_B, pb->m22, NC) | up(e, e->d_C, pb->m12, NC) |
       up(e, e->d_V, pb->svel, NC);
  for (DBuf* b : {&e->d_a, &e->d_b, &e->d_c, &e->d_fun, &e->d_f2, &e->d_disx, &e->d_disy})
    r |= up(e, *b, (double*)nullptr, NC);
  r |= up(e, e->d_f32, (float*)nullptr, 6 * NC) | up(e, e->d_isv, (double*)nullptr, 2 * NC);
  r |= up(e, e->d_p4a, (float4*)nullptr, 2 * NC);
  r |= up(e, e->d_pidx, pb->pidx, ns) | up(e, e->d_srcx, pb->srcx, ns) |
       up(e, e->d_srcy, pb->srcy, ns) | up(e, e->d_rec_off, pb->rec_off, ns) |
       up(e, e->d_nrec, pb->nrec, ns);
  r |= up(e, e->d_recx, pb->recx, nrec_total) | up(e, e->d_recy, pb->recy, nrec_total) |
       up(e, e->d_tt, pb->tt, nrec_total) | up(e, e->d_weight, pb->weight, nrec_total) |
       up(e, e->d_path, pb->path, nrec_total);
  r |= up(e, e->d_order, e->order.data(), ns) | up(e, e->d_plist_off, e->plist_off.data(), np + 1) |
       up(e, e->d_plist, e->plist.data(), ns) | up(e, e->d_kslot, e->kslot.data(), ns) |
       up(e, e->d_goff, e->goff.data(), np) | up(e, e->d_nx, e->nx.data(), np) |
       up(e, e->d_ny, e->ny.data(), np);
  // outputs
  r |= up(e, e->d_tekio, (double*)nullptr, nrec_total) | up(e, e->d_wgt, (double*)nullptr, nrec_total) |
       up(e, e->d_ttfwd, (double*)nullptr, std::max(1, pb->npath)) |
       up(e, e->d_chis, (double*)nullptr, ns) | up(e, e->d_chi, (double*)nullptr, 1) |
       up(e, e->d_kc, (double*)nullptr, e->kslot_total) |
       up(e, e->d_kcd, (double*)nullptr, e->kslot_total) | up(e, e->d_adj, (double*)nullptr, NC) |
       up(e, e->d_adjd, (double*)nullptr, NC) | up(e, e->d_status, (int*)nullptr, ns) |
       up(e, e->d_fit, (int*)nullptr, ns) | up(e, e->d_ait, (int*)nullptr, ns) |
       up(e, e->d_fupd, (double*)nullptr, ns) | up(e, e->d_aupd, (double*)nullptr, ns) |
       up(e, e->d_queue, (int*)nullptr, kTeamClasses);
  if (r & SURFATT_CUDA_ERROR) return SURFATT_CUDA_ERROR;
  if (r) return SURFATT_OOM;
  // per-period descriptors
  e->periods.resize(np);
  for (int p = 0; p < np; ++p) {
    PeriodDev& P = e->periods[p];
    const long long g = e->goff[p];
    P.nx = e->nx[p];
    P.ny = e->ny[p];
    P.lonlat = 1;
    const double* xg = pb->xgrid + e->xoff[p];
    const double* yg = pb->ygrid + e->yoff[p];
    P.dx = xg[1] / 180.0 * PI_S - xg[0] / 180.0 * PI_S;
    P.dy = yg[1] / 180.0 * PI_S - yg[0] / 180.0 * PI_S;
    P.xs = e->d_xs.as<double>() + e->xoff[p];
    P.ys = e->d_ys.as<double>() + e->yoff[p];
    P.xdeg = e->d_xdeg.as<double>() + e->xoff[p];
    P.ydeg = e->d_ydeg.as<double>() + e->yoff[p];
    P.cosy = e->d_cosy.as<double>() + e->yoff[p];
    P.siny = e->d_siny.as<double>() + e->yoff[p];
    P.a = e->d_a.as<double>() + g;
    P.b = e->d_b.as<double>() + g;
    P.c = e->d_c.as<double>() + g;
    P.fun = e->d_fun.as<double>() + g;
    P.f2 = e->d_f2.as<double>() + g;
    P.disx = e->d_disx.as<double>() + g;
    P.disy = e->d_disy.as<double>() + g;
    P.svel = e->d_V.as<double>() + g;
    P.goff = g;
    P.f32 = e->d_f32.as<float>() + 6 * g;
    P.isv = e->d_isv.as<double>() + 2 * g;
    P.p4a = e->d_p4a.as<float4>() + 2 * g;
    P.p4b = P.p4a + 1;
  }
  r = up(e, e->d_periods, e->periods.data(), np);
  if (r) return (surfatt_status_t)r;
  r = run_prep_all(e);
  if (r) return (surfatt_status_t)r;
  // Captured evaluations hold the problem's sizes: capture again only when
  // they change (buffers that had to grow have moved `gen` already).
  std::vector<long long> sig = {np, ns, pb->npath, nrec_total, e->ncell, e->kslot_total};
  for (int p = 0; p < np; ++p) {
    sig.push_back(e->nx[p]);
    sig.push_back(e->ny[p]);
    sig.push_back(e->goff[p]);
  }
  if (sig != e->shape_sig) {
    ++e->gen;
    e->shape_sig = sig;
  }
  e->loaded = true;
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_update_velocity(surfatt_engine_t* e, const double* svel) {
  if (!e || !e->loaded || !svel) return SURFATT_BAD_ARG;
  CK(cudaSetDevice(e->device));
  CK(cudaMemcpyAsync(e->d_V.p, svel, (size_t)e->ncell * sizeof(double), cudaMemcpyHostToDevice,
                     e->st));
  return (surfatt_status_t)run_prep_all(e);
}

}  // extern "C"

namespace {
// Enqueue one evaluation.  With `graph`, the evaluation (resets, solve
// kernel, kernel sums, misfit sum) is captured once into an executable graph
// per (mode, precision) and replayed by one cudaGraphLaunch afterwards.
int engine_enqueue(surfatt_engine* e, int mode, int prec, const KernelChoice& force,
                   bool graph = false) {
  CK(cudaSetDevice(e->device));
  EvalShape sh;
  sh.from_grids(e->nx.data(), e->ny.data(), e->goff.data(), e->nperiod, e->nsolve, e->npath,
                e->pidx.data());
  LaunchPlan plan;
  int r = plan_evaluation(sh, prec, e->device, 0, &plan, force);
  if (r) return (surfatt_status_t)r;
  r = eng_ensure(e, e->d_ws, (size_t)plan_ws_doubles(plan, e->nsolve) * sizeof(double));
  if (r) return (surfatt_status_t)r;
  e->grid = plan.grid;
  e->per_sm = plan.per_sm;
  e->last_block = plan.block;
  e->last_smem = plan.smem;
  e->last_kind = plan.kind;
  e->last_pf = plan.pf;
  EvalDev dev;
  BatchArgs& A = dev.args;
  A.periods = e->d_periods.as<PeriodDev>();
  A.nsolve = e->nsolve;
  A.order = e->d_order.as<int>();
  A.pidx = e->d_pidx.as<int>();
  A.srcx = e->d_srcx.as<double>();
  A.srcy = e->d_srcy.as<double>();
  A.rec_off = e->d_rec_off.as<int>();
  A.nrec = e->d_nrec.as<int>();
  A.recx = e->d_recx.as<double>();
  A.recy = e->d_recy.as<double>();
  A.tt = e->d_tt.as<double>();
  A.weight = e->d_weight.as<double>();
  A.path = e->d_path.as<int>();
  A.kslot = e->d_kslot.as<long long>();
  A.tekio = e->d_tekio.as<double>();
  A.wgt_eff = e->d_wgt.as<double>();
  A.tt_fwd = e->d_ttfwd.as<double>();
  A.chi = e->d_chis.as<double>();
  A.kcontrib = e->d_kc.as<double>();
  A.kcontrib_den = e->d_kcd.as<double>();
  A.status = e->d_status.as<int>();
  A.fwd_iters = e->d_fit.as<int>();
  A.adj_iters = e->d_ait.as<int>();
  A.fwd_updates = e->d_fupd.as<double>();
  A.adj_updates = e->d_aupd.as<double>();
  A.Tout = nullptr;
  if (e->keep_fields) {
    r = eng_ensure(e, e->d_T, (size_t)std::max(1LL, e->kslot_total) * sizeof(double));
    if (r) return r;
    A.Tout = e->d_T.as<double>();
  }
  A.hold_solve = e->hold_solve;
  A.item_wait_limit = e->item_wait_limit;
  if (e->profile) {
    r = eng_ensure(e, e->d_phase, PH_COUNT * sizeof(unsigned long long));
    if (r) return r;
    A.phase_cycles = e->d_phase.as<unsigned long long>();
  }
  dev.plist_off = e->d_plist_off.as<int>();
  dev.plist = e->d_plist.as<int>();
  dev.goff = e->d_goff.as<long long>();
  dev.nx = e->d_nx.as<int>();
  dev.ny = e->d_ny.as<int>();
  dev.chi_total = e->d_chi.as<double>();
  dev.adj_s = e->d_adj.as<double>();
  dev.adj_density = e->d_adjd.as<double>();
  if (graph) {
    auto& g = e->graphs[mode][prec];
    if (!g.exec || g.gen != e->gen || g.kind != plan.kind || g.pf != plan.pf ||
        g.grid != plan.grid) {
      if (g.exec) cudaGraphExecDestroy(g.exec);
      g = surfatt_engine::Captured();
      cudaGraph_t gr = nullptr;
      CK(cudaStreamBeginCapture(e->st, cudaStreamCaptureModeRelaxed));
      const int n = enqueue_evaluation(sh, dev, plan, mode, prec, e->d_ws.as<double>(),
                                       e->d_queue.as<int>(), e->st, e->evk0, e->evk1, &e->cs);
      const cudaError_t ce = cudaStreamEndCapture(e->st, &gr);
      if (n < 0 || ce != cudaSuccess) {
        if (gr) cudaGraphDestroy(gr);
        cudaGetLastError();
        return n < 0 ? -n : SURFATT_CUDA_ERROR;
      }
      const cudaError_t ci = cudaGraphInstantiate(&g.exec, gr, 0);
      cudaGraphDestroy(gr);
      if (ci != cudaSuccess) {
        g.exec = nullptr;
        cudaGetLastError();
        return SURFATT_CUDA_ERROR;
      }
      g.gen = e->gen;
      g.kind = plan.kind;
      g.pf = plan.pf;
      g.grid = plan.grid;
      g.launches = n;
    }
    CK(cudaEventRecord(e->ev0, e->st));
    CK(cudaGraphLaunch(g.exec, e->st));
    CK(cudaEventRecord(e->ev1, e->st));
    e->launches = g.launches;
  } else {
    CK(cudaEventRecord(e->ev0, e->st));
    const int n = enqueue_evaluation(sh, dev, plan, mode, prec, e->d_ws.as<double>(),
                                     e->d_queue.as<int>(), e->st, e->evk0, e->evk1, &e->cs);
    if (n < 0) return -n;
    CK(cudaEventRecord(e->ev1, e->st));
    e->launches = n;
  }
  e->ran = true;
  e->last_mode = mode;
  return SURFATT_OK;
}
}  // namespace

extern "C" {

surfatt_status_t surfatt_engine_run(surfatt_engine_t* e, surfatt_mode_t mode,
                                    surfatt_precision_t prec) {
  if (!e || !e->loaded) return SURFATT_BAD_ARG;
  if (mode != SURFATT_MODE_FORWARD && mode != SURFATT_MODE_2D && mode != SURFATT_MODE_3D)
    return SURFATT_BAD_ARG;
  if (prec != SURFATT_PREC_FP64 && prec != SURFATT_PREC_FP32) return SURFATT_BAD_ARG;
  const int p = prec == SURFATT_PREC_FP64 ? 0 : 1;
  return (surfatt_status_t)engine_enqueue(e, mode, p, e->tuned[p],
                                          e->use_graphs);
}

surfatt_status_t surfatt_engine_set_kernel(surfatt_engine_t* e, surfatt_precision_t prec,
                                          int kind, int variant) {
  if (!e) return SURFATT_BAD_ARG;
  if (prec != SURFATT_PREC_FP64 && prec != SURFATT_PREC_FP32) return SURFATT_BAD_ARG;
  const int p = prec == SURFATT_PREC_FP64 ? 0 : 1;
  if (p == 0 && kind != -1 && kind != KK_FP64) return SURFATT_BAD_ARG;
  if (p == 1 && kind != -1 && kind != KK_FP32_BLOCK && kind != KK_FP32_WARP)
    return SURFATT_BAD_ARG;
  if (variant < -1 || variant >= fp32w_variant_count()) return SURFATT_BAD_ARG;
  e->tuned[p] = KernelChoice{kind, variant};
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_set_profile(surfatt_engine_t* e, int enable) {
  if (!e) return SURFATT_BAD_ARG;
  e->profile = enable != 0;
  ++e->gen;  // the kernel arguments change
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_phase_cycles(surfatt_engine_t* e, double* cycles) {
  if (!e || !e->ran || !cycles || !e->profile || !e->d_phase.p) return SURFATT_BAD_ARG;
  CK(cudaSetDevice(e->device));
  CK(cudaStreamSynchronize(e->st));
  unsigned long long c[PH_COUNT];
  CK(cudaMemcpy(c, e->d_phase.p, sizeof(c), cudaMemcpyDeviceToHost));
  for (int i = 0; i < PH_COUNT; ++i) cycles[i] = (double)c[i];
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_set_graphs(surfatt_engine_t* e, int enable) {
  if (!e) return SURFATT_BAD_ARG;
  CK(cudaSetDevice(e->device));
  CK(cudaStreamSynchronize(e->st));
  e->use_graphs = enable != 0;
  if (!e->use_graphs) e->drop_graphs();
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_autotune(surfatt_engine_t* e, surfatt_mode_t mode,
                                         surfatt_precision_t prec, int* kind, int* variant,
                                         double* best_ms) {
  if (!e || !e->loaded) return SURFATT_BAD_ARG;
  if (prec != SURFATT_PREC_FP64 && prec != SURFATT_PREC_FP32) return SURFATT_BAD_ARG;
  const int p = prec == SURFATT_PREC_FP64 ? 0 : 1;
  EvalShape sh;
  sh.from_grids(e->nx.data(), e->ny.data(), e->goff.data(), e->nperiod, e->nsolve, e->npath,
                e->pidx.data());
  double best = 1e300;
  KernelChoice bc;
  // one warm-up and one timed evaluation of a candidate
  auto time_one = [&](const KernelChoice& c) -> int {
    float ms = 0.f;
    int r = engine_enqueue(e, mode, p, c);
    if (r) return r;
    r = engine_enqueue(e, mode, p, c);
    if (r) return r;
    CK(cudaEventSynchronize(e->ev1));
    CK(cudaEventElapsedTime(&ms, e->evk0, e->evk1));
    if (ms < best) {
      best = ms;
      bc = c;
    }
    return SURFATT_OK;
  };
  for (const auto& c : plan_candidates(sh, p)) {
    const int r = time_one(c);
    if (r) return (surfatt_status_t)r;
  }
  e->tuned[p] = bc;
  if (kind) *kind = bc.kind;
  if (variant) *variant = bc.variant;
  if (best_ms) *best_ms = best;
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_sync(surfatt_engine_t* e) {
  if (!e || !e->ran) return SURFATT_BAD_ARG;
  CK(cudaSetDevice(e->device));
  CK(cudaStreamSynchronize(e->st));
  std::vector<int> st(std::max(1, e->nsolve));
  if (e->nsolve)
    CK(cudaMemcpy(st.data(), e->d_status.p, e->nsolve * sizeof(int), cudaMemcpyDeviceToHost));
  for (int s = 0; s < e->nsolve; ++s)
    if (st[s] != SURFATT_OK) return (surfatt_status_t)st[s];
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_results(surfatt_engine_t* e, surfatt_result_t* out) {
  if (!e || !e->ran || !out) return SURFATT_BAD_ARG;
  CK(cudaSetDevice(e->device));
  const size_t NC = (size_t)e->ncell;
  if (out->adj_s) {
    if (e->last_mode >= 2)
      CK(cudaMemcpyAsync(out->adj_s, e->d_adj.p, NC * sizeof(double), cudaMemcpyDeviceToHost, e->st));
    else
      std::memset(out->adj_s, 0, NC * sizeof(double));
  }
  if (out->adj_density) {
    if (e->last_mode == 3)
      CK(cudaMemcpyAsync(out->adj_density, e->d_adjd.p, NC * sizeof(double),
                         cudaMemcpyDeviceToHost, e->st));
    else
      std::memset(out->adj_density, 0, NC * sizeof(double));
  }
  if (out->chi) CK(cudaMemcpyAsync(out->chi, e->d_chi.p, sizeof(double), cudaMemcpyDeviceToHost, e->st));
  if (out->tt_fwd && e->npath)
    CK(cudaMemcpyAsync(out->tt_fwd, e->d_ttfwd.p, e->npath * sizeof(double), cudaMemcpyDeviceToHost, e->st));
  if (out->status && e->nsolve)
    CK(cudaMemcpyAsync(out->status, e->d_status.p, e->nsolve * sizeof(int), cudaMemcpyDeviceToHost, e->st));
  if (out->fwd_iters && e->nsolve)
    CK(cudaMemcpyAsync(out->fwd_iters, e->d_fit.p, e->nsolve * sizeof(int), cudaMemcpyDeviceToHost, e->st));
  if (out->adj_iters && e->nsolve)
    CK(cudaMemcpyAsync(out->adj_iters, e->d_ait.p, e->nsolve * sizeof(int), cudaMemcpyDeviceToHost, e->st));
  CK(cudaStreamSynchronize(e->st));
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_timing(surfatt_engine_t* e, double* total_ms,
                                       double* solve_kernel_ms, int* launches) {
  if (!e || !e->ran) return SURFATT_BAD_ARG;
  CK(cudaSetDevice(e->device));
  CK(cudaEventSynchronize(e->ev1));
  float a = 0, b = 0;
  CK(cudaEventElapsedTime(&a, e->ev0, e->ev1));
  CK(cudaEventElapsedTime(&b, e->evk0, e->evk1));
  if (total_ms) *total_ms = a;
  if (solve_kernel_ms) *solve_kernel_ms = b;
  if (launches) *launches = e->launches;
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_smooth(surfatt_engine_t* e, double sigma, double* ker_s) {
  if (!e || !e->ran || e->last_mode < 2) return SURFATT_BAD_ARG;
  CK(cudaSetDevice(e->device));
  if (sigma != e->sm_sigma) {
    e->sm_sigma = -1.0;
    const std::vector<double> sig(e->nperiod, sigma);
    if (smooth_plan(e->nperiod, e->nx.data(), e->ny.data(), e->goff.data(), nullptr,
                    e->xoff.data(), e->yoff.data(), e->hx.data(), e->hy.data(), sig.data(),
                    &e->smplan) != ST_OK)
      return SURFATT_BAD_ARG;
    const SmoothPlan& P = e->smplan;
    int r = up(e, e->d_ker, (double*)nullptr, (size_t)e->ncell);
    r |= up(e, e->d_smtab, (double*)nullptr, (size_t)P.table_doubles);
    r |= up(e, e->d_smnyw, P.nyw.data(), (size_t)P.nyw_count);
    r |= up(e, e->d_smper, P.per.data(), P.per.size());
    if (r) return SURFATT_OOM;
  }
  SmoothArgs A{e->d_smper.as<SmoothPeriod>(), e->nperiod, e->d_xdeg.as<double>(),
               e->d_ydeg.as<double>(), e->d_smnyw.as<int>(), e->d_adj.as<double>(),
               e->d_ker.as<double>(), e->d_smtab.as<double>(), e->smplan.nodes};
  CK(cudaEventRecord(e->evs0, e->st));
  e->sm_launches = 1;
  if (sigma != e->sm_sigma) {  // the table depends on the grids and sigma only
    launch_smooth_table(A, e->smplan, e->st);
    CK(cudaGetLastError());
    e->sm_sigma = sigma;
    e->sm_launches = 2;
  }
  launch_smooth_apply(A, e->smplan, e->st);
  CK(cudaGetLastError());
  CK(cudaEventRecord(e->evs1, e->st));
  e->smoothed = true;
  if (ker_s) {
    CK(cudaMemcpyAsync(ker_s, e->d_ker.p, (size_t)e->ncell * sizeof(double),
                       cudaMemcpyDeviceToHost, e->st));
    CK(cudaStreamSynchronize(e->st));
  }
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_smooth_timing(surfatt_engine_t* e, double* kernel_ms,
                                              double* taps, int* launches) {
  if (!e || !e->smoothed) return SURFATT_BAD_ARG;
  CK(cudaSetDevice(e->device));
  CK(cudaEventSynchronize(e->evs1));
  float a = 0;
  CK(cudaEventElapsedTime(&a, e->evs0, e->evs1));
  if (kernel_ms) *kernel_ms = a;
  if (taps) *taps = e->smplan.taps;
  if (launches) *launches = e->sm_launches;
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_launch_config(surfatt_engine_t* e, int* grid, int* block,
                                              int* blocks_per_sm, size_t* smem_bytes) {
  if (!e || !e->ran) return SURFATT_BAD_ARG;
  if (grid) *grid = e->grid;
  if (block) *block = e->last_block;
  if (blocks_per_sm) *blocks_per_sm = e->per_sm;
  if (smem_bytes) *smem_bytes = e->last_smem;
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_kernel_variant(surfatt_engine_t* e, int* kind, int* pf) {
  if (!e || !e->ran) return SURFATT_BAD_ARG;
  if (kind) *kind = e->last_kind;
  if (pf) *pf = e->last_pf;
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_set_keep_fields(surfatt_engine_t* e, int enable) {
  if (!e) return SURFATT_BAD_ARG;
  e->keep_fields = enable != 0;
  ++e->gen;  // the kernel arguments change
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_fields(surfatt_engine_t* e, double* T) {
  if (!e || !e->ran || !e->keep_fields || !T || !e->d_T.p) return SURFATT_BAD_ARG;
  CK(cudaSetDevice(e->device));
  CK(cudaStreamSynchronize(e->st));
  if (e->kslot_total > 0)
    CK(cudaMemcpy(T, e->d_T.p, (size_t)e->kslot_total * sizeof(double), cudaMemcpyDeviceToHost));
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_test_hold(surfatt_engine_t* e, int solve, int wait_polls) {
  if (!e || solve < -1 || wait_polls < 0) return SURFATT_BAD_ARG;
  e->hold_solve = solve;
  e->item_wait_limit = wait_polls;
  ++e->gen;  // the kernel arguments change
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_device_results(surfatt_engine_t* e, double** adj_s,
                                               double** adj_density, double** tt_fwd,
                                               double** chi, void** stream) {
  if (!e || !e->ran) return SURFATT_BAD_ARG;
  if (adj_s) *adj_s = e->last_mode >= 2 ? static_cast<double*>(e->d_adj.p) : nullptr;
  if (adj_density) *adj_density = e->last_mode == 3 ? static_cast<double*>(e->d_adjd.p) : nullptr;
  if (tt_fwd) *tt_fwd = e->npath ? static_cast<double*>(e->d_ttfwd.p) : nullptr;
  if (chi) *chi = static_cast<double*>(e->d_chi.p);
  if (stream) *stream = static_cast<void*>(e->st);
  return SURFATT_OK;
}

surfatt_status_t surfatt_engine_work(surfatt_engine_t* e, double* fwd, double* adj) {
  if (!e || !e->ran) return SURFATT_BAD_ARG;
  CK(cudaSetDevice(e->device));
  CK(cudaStreamSynchronize(e->st));
  std::vector<double> f(std::max(1, e->nsolve)), a(std::max(1, e->nsolve));
  if (e->nsolve) {
    CK(cudaMemcpy(f.data(), e->d_fupd.p, e->nsolve * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(a.data(), e->d_aupd.p, e->nsolve * sizeof(double), cudaMemcpyDeviceToHost));
  }
  double sf = 0, sa = 0;
  for (int s = 0; s < e->nsolve; ++s) {
    sf += f[s];
    sa += a[s];
  }
  if (fwd) *fwd = sf;
  if (adj) *adj = sa;
  return SURFATT_OK;
}

}  // extern "C"
