// batch_tail.cuh -- the steps of a batched solve after its forward sweeps
// (shared by the FP64 and FP32 solve kernels): receiver interpolation,
// misfit, outlier weights, adjoint sources, adjoint sweeps, mask and the
// per-solve kernel contribution.
#pragma once
#include "kernels.cuh"
#include "solver_fp64.cuh"

namespace sgb {

// Receiver times (interp2 on the caller's degree grid), misfit and outlier
// weights of solve s (src/measadj.f90:71-72, 82-84).  Leaves the block
// synchronised; a receiver outside the grid sets sh.flag.
__device__ inline void tail_receivers(const BatchArgs& A, const PeriodDev& P, int s,
                                      const double* T, SolveShared& sh) {
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  const int r0 = A.rec_off[s], nr = A.nrec[s];
  // receiver times (interp2 on the caller's degree grid)
  for (int r = threadIdx.x; r < nr; r += blockDim.x) {
    double v = 0.0;
    if (!interp2(P.xdeg, nx, P.ydeg, ny, T, A.recx[r0 + r], A.recy[r0 + r], &v))
      atomicExch(&sh.flag, ST_BAD_ARG);
    A.tekio[r0 + r] = v;
    A.tt_fwd[A.path[r0 + r]] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // chi = 0.5*sum(weight*(tekio-tt)**2) (src/measadj.f90:72), then the
    // outlier weights (:82-84) for the adjoint sources.
    double ssum = 0;
    for (int r = 0; r < nr; ++r) {
      const double d = A.tekio[r0 + r] - A.tt[r0 + r];
      ssum = ssum + A.weight[r0 + r] * (d * d);
    }
    A.chi[s] = 0.5 * ssum;
    for (int r = 0; r < nr; ++r) {
      double w = A.weight[r0 + r];
      if (fabs(A.tekio[r0 + r] - A.tt[r0 + r]) / A.tt[r0 + r] > 0.5) w = 0.;
      A.wgt_eff[r0 + r] = w;
    }
  }
  if (A.Tout)
    for (size_t k = threadIdx.x; k < N; k += blockDim.x) A.Tout[A.kslot[s] + k] = T[k];
  __syncthreads();
}

// Steps of the plain FP64 solve after its forward sweeps:
// T -> receivers -> misfit -> adjoint(s) -> mask -> kernel slot.
__device__ inline void solve_tail(const BatchArgs& A, const PeriodDev& P, int s,
                                  const double* T, const AdjWs& aw, SolveShared& sh,
                                  int fwd_status, int fwd_iters) {
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  const int r0 = A.rec_off[s], nr = A.nrec[s];
  tail_receivers(A, P, s, T, sh);
  int st = fwd_status;
  if (sh.flag != ST_OK && st == ST_OK) st = sh.flag;
  int aiters = 0;
  if (A.mode >= 2) {
    const int nf = A.mode == 3 ? 2 : 1;
    for (int f = 0; f < nf; ++f)
      for (size_t k = threadIdx.x; k < N; k += blockDim.x) aw.delta[f][k] = 0.0;
    __syncthreads();
    if (threadIdx.x == 0) {
      // sourceAdj = weight*(tekio-tt) (:88) and -1.0*weight (:102)
      int e = ST_OK;
      for (int f = 0; f < nf && e == ST_OK; ++f) {
        const double* rx = A.recx + r0;
        const double* ry = A.recy + r0;
        // splat one receiver at a time in receiver order
        for (int r = 0; r < nr && e == ST_OK; ++r) {
          const double w = A.wgt_eff[r0 + r];
          const double sv = f == 0 ? w * (A.tekio[r0 + r] - A.tt[r0 + r]) : -1.0 * w;
          e = adj_splat(P, aw.delta[f], 1, rx + r, ry + r, nullptr, sv);
        }
      }
      if (e != ST_OK) sh.flag = e;
    }
    __syncthreads();
    if (sh.flag != ST_OK && st == ST_OK) st = sh.flag;
    adj_setup(P, aw, nf);
    int its[2] = {0, 0}, sts[2] = {ST_OK, ST_OK};
    adj_sweeps(P, aw, nf, sh, its, sts);
    aiters = its[0] > its[1] ? its[0] : its[1];
    for (int f = 0; f < nf; ++f)
      if (sts[f] != ST_OK && st == ST_OK) st = sts[f];
    const double x0 = A.srcx[s], y0 = A.srcy[s];
    for (int f = 0; f < nf; ++f) apply_mask(P, aw.Ta[f], x0, y0);
    // kernel contribution: adj / svel**k  (src/tomo2d.f90:155, src/acqui.f90:314-315)
    double* ks = A.kcontrib + A.kslot[s];
    double* kd = A.mode == 3 ? A.kcontrib_den + A.kslot[s] : nullptr;
    for (size_t k = threadIdx.x; k < N; k += blockDim.x) {
      const double v = P.svel[k];
      if (A.mode == 3) {
        ks[k] = aw.Ta[0][k] / (v * v * v);
        kd[k] = aw.Ta[1][k] / (v * v * v);
      } else {
        ks[k] = aw.Ta[0][k] / (v * v);
      }
    }
    if (A.adj_updates && threadIdx.x == 0)
      A.adj_updates[s] = (double)(its[0] + its[1]) * 4.0 * (nx - 2) * (ny - 2);
  }
  if (threadIdx.x == 0) {
    A.status[s] = st;
    A.fwd_iters[s] = fwd_iters;
    A.adj_iters[s] = aiters;
  }
  __syncthreads();
}

// Zero outputs of a solve that could not run (source on boundary / outside).
__device__ inline void solve_fail(const BatchArgs& A, const PeriodDev& P, int s, int st) {
  const size_t N = (size_t)P.nx * P.ny;
  const int r0 = A.rec_off[s], nr = A.nrec[s];
  for (int r = threadIdx.x; r < nr; r += blockDim.x) {
    A.tekio[r0 + r] = 0.0;
    A.wgt_eff[r0 + r] = 0.0;
    A.tt_fwd[A.path[r0 + r]] = 0.0;
  }
  if (A.mode >= 2)
    for (size_t k = threadIdx.x; k < N; k += blockDim.x) {
      A.kcontrib[A.kslot[s] + k] = 0.0;
      if (A.mode == 3) A.kcontrib_den[A.kslot[s] + k] = 0.0;
    }
  if (A.Tout)
    for (size_t k = threadIdx.x; k < N; k += blockDim.x) A.Tout[A.kslot[s] + k] = 0.0;
  if (threadIdx.x == 0) {
    A.chi[s] = 0.0;
    A.status[s] = st;
    A.fwd_iters[s] = 0;
    A.adj_iters[s] = 0;
    if (A.fwd_updates) A.fwd_updates[s] = 0;
    if (A.adj_updates) A.adj_updates[s] = 0;
  }
  __syncthreads();
}

}  // namespace sgb
