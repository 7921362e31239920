// kernels_fp32.cu -- the batched solve with the factored unknown tau = T/T0
// swept in FP32.
//
// What stays FP64: the analytic spherical T0 and its gradient (computed in
// FP64, then the per-cell sweep coefficients are rounded once), the
// convergence decision (sum and max of |dtau|*T0 accumulated in FP64 from
// the FP32 iterates), the travel times T = tau*T0, receiver interpolation,
// misfit, adjoint sources, the adjoint sweeps and the kernel sums.
//
// The FP32 sweep does not evaluate the reference's quadratic in tau
// directly: with tau = tau_X + delta (tau_X the upwind x neighbour) the
// terms px*tau + qx = T0x*tau_X + px*delta and
// py*tau + qy = T0y*tau_X - sY*cy*(tau_X - tau_Y) + py*delta carry no
// cancellation between the O(T0/dx) terms, so delta (and tau) keep FP32
// relative accuracy.  It is the same local equation and the same candidate
// set (causal two-sided roots, admissible one-sided roots, min) as
// FSM_UW_PS_lonlat_2d (src/eikon_solver_2d.f90:904-1079).
#include "kernels.cuh"
#include "solver_fp64.cuh"
#include "batch_tail.cuh"

namespace sgb {

enum F32Const {
  KF_CX = 0, KF_CY, KF_T0X, KF_T0Y,
  KF_A,                 // eqn_a per case (4)
  KF_IA = KF_A + 4,     // 1/eqn_a (4)
  KF_BX = KF_IA + 4,    // a*px - c*py (4)
  KF_BY = KF_BX + 4,    // b*py - c*px (4)
  KF_IP = KF_BY + 4,    // 1/(T0x+cx), 1/(T0x-cx), 1/(T0y+cy), 1/(T0y-cy)
  KF_a = KF_IP + 4, KF_b, KF_c, KF_F2, KF_DX, KF_DY,
  KF_COUNT
};

// Workspace per solve slot (in doubles): FP64 part (tau_old not needed:
// T0, T, adjoint fields) + FP32 part (tau, tau_old, constants).
long long batch_fp32_ws_doubles(long long N) {
  const long long f64 = 2 * N + (long long)(KA_COUNT + 6) * N;  // T0, T, adjoint
  const long long f32 = (2 + (long long)KF_COUNT) * N;          // floats
  return f64 + (f32 + 1) / 2 + 8;
}

struct F32Layout {
  double* T0;
  double* T;
  AdjWs aw;
  float* tau;
  float* tau_old;
  float* K;
};

__device__ inline F32Layout carve32(double* base, size_t N) {
  F32Layout L;
  L.T0 = base;
  L.T = base + N;
  L.aw.T = L.T;
  L.aw.K = base + 2 * N;
  double* f = base + 2 * N + KA_COUNT * N;
  L.aw.delta[0] = f;
  L.aw.delta[1] = f + N;
  L.aw.Ta[0] = f + 2 * N;
  L.aw.Ta[1] = f + 3 * N;
  L.aw.old[0] = f + 4 * N;
  L.aw.old[1] = f + 5 * N;
  float* g = reinterpret_cast<float*>(f + 6 * N);
  L.tau = g;
  L.tau_old = g + N;
  L.K = g + 2 * N;
  return L;
}

// Setup: FP64 T0 (same formulas as the plain path), FP32 constants.
__device__ inline void f32_setup(const PeriodDev& P, double x0, double y0, const F32Layout& L,
                                 SolveShared& sh) {
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  if (threadIdx.x == 0) {
    sh.status = ST_OK;
    float r1 = 0.f, r2 = 0.f;
    const int i0 = locate_cell(P.xs, nx - 1, P.dx, x0, &r1);
    const int j0 = locate_cell(P.ys, ny - 1, P.dy, y0, &r2);
    if (i0 < 0 || j0 < 0) {
      sh.status = ST_BAD_ARG;
    } else {
      float w00 = (1 - r1) * (1 - r2), w01 = (1 - r1) * r2, w10 = r1 * (1 - r2), w11 = r1 * r2;
      const size_t k00 = i0 + (size_t)nx * j0;
      sh.fun0 = (double)w00 * P.fun[k00] + (double)w01 * P.fun[k00 + nx] +
                (double)w10 * P.fun[k00 + 1] + (double)w11 * P.fun[k00 + nx + 1];
    }
    int a0 = nx, a1 = -1, b0 = ny, b1 = -1;
    for (int i = 0; i < nx; ++i)
      if (fabs((P.xs[i] - x0) / P.dx) <= 1.0) { a0 = min(a0, i); a1 = max(a1, i); }
    for (int j = 0; j < ny; ++j)
      if (fabs((P.ys[j] - y0) / P.dy) <= 1.0) { b0 = min(b0, j); b1 = max(b1, j); }
    sh.box = Box{a0, a1, b0, b1};
    if (sh.status == ST_OK && a0 <= a1 && b0 <= b1 &&
        (a0 == 0 || a1 == nx - 1 || b0 == 0 || b1 == ny - 1))
      sh.status = ST_SOURCE_ON_BOUNDARY;
  }
  __syncthreads();
  if (sh.status != ST_OK) return;
  const double fun0 = sh.fun0;
  const Box box = sh.box;
  const double cy0 = cos(y0), sy0 = sin(y0);
  float* K = L.K;
  for (size_t k = threadIdx.x; k < N; k += blockDim.x) {
    const int i = (int)(k % nx), j = (int)(k / nx);
    const double cyy = P.cosy[j], syy = P.siny[j];
    const double cdx = cos(P.xs[i] - x0), sdx = sin(P.xs[i] - x0);
    const double tmp = syy * sy0 + cyy * cy0 * cdx;
    double cl = tmp < 1.0 ? tmp : 1.0;
    cl = cl > -1.0 ? cl : -1.0;
    const double t0 = acos(cl) * R_EARTH * fun0;
    double t0x = 0, t0y = 0;
    if (t0 != 0) {
      const double rs = 1.0 / sqrt(1 - tmp * tmp);
      t0x = -(rs * cyy * cy0 * (-1.0) * sdx * R_EARTH * fun0);
      t0y = -(rs * (cyy * sy0 - syy * cy0 * cdx) * R_EARTH * fun0);
    }
    L.T0[k] = t0;
    L.tau[k] = box.has(i, j) ? 1.0f : 10.0f;
    const double a = P.a[k], b = P.b[k], c = P.c[k];
    const double cx = t0 / P.dx, cy = t0 / P.dy;
    K[KF_CX * N + k] = (float)cx;
    K[KF_CY * N + k] = (float)cy;
    K[KF_T0X * N + k] = (float)t0x;
    K[KF_T0Y * N + k] = (float)t0y;
    const double pxm = t0x + cx, pxp = t0x - cx, pym = t0y + cy, pyp = t0y - cy;
#pragma unroll
    for (int cs = 0; cs < 4; ++cs) {
      const double px = cs < 2 ? pxm : pxp;
      const double py = (cs == 0 || cs == 2) ? pym : pyp;
      const double ea = a * (px * px) + b * (py * py) - 2 * c * px * py;
      K[(KF_A + cs) * N + k] = (float)ea;
      K[(KF_IA + cs) * N + k] = (float)(1.0 / ea);
      K[(KF_BX + cs) * N + k] = (float)(a * px - c * py);
      K[(KF_BY + cs) * N + k] = (float)(b * py - c * px);
    }
    K[(KF_IP + 0) * N + k] = (float)(1.0 / pxm);
    K[(KF_IP + 1) * N + k] = (float)(1.0 / pxp);
    K[(KF_IP + 2) * N + k] = (float)(1.0 / pym);
    K[(KF_IP + 3) * N + k] = (float)(1.0 / pyp);
    K[KF_a * N + k] = (float)a;
    K[KF_b * N + k] = (float)b;
    K[KF_c * N + k] = (float)c;
    K[KF_F2 * N + k] = (float)P.f2[k];
    K[KF_DX * N + k] = (float)P.disx[k];
    K[KF_DY * N + k] = (float)P.disy[k];
  }
  __syncthreads();
}

// FP32 visit of cell k in the tau = tau_nb + delta form.
__device__ __forceinline__ float f32_update(const float* __restrict__ K, size_t N, size_t k, int i,
                                            int j, int nx, int ny, const float* tau,
                                            const double* __restrict__ T0d, float t) {
  const bool hw = i > 0, he = i < nx - 1, hs = j > 0, hn = j < ny - 1;
  const float cy = K[KF_CY * N + k];
  const float t0x = K[KF_T0X * N + k], t0y = K[KF_T0Y * N + k];
  const float a = K[KF_a * N + k], b = K[KF_b * N + k], c = K[KF_c * N + k];
  const float f2 = K[KF_F2 * N + k];
  const float tw = hw ? tau[k - 1] : 0.f, te = he ? tau[k + 1] : 0.f;
  const float ts = hs ? tau[k - nx] : 0.f, tn = hn ? tau[k + nx] : 0.f;
#pragma unroll
  for (int cs = 0; cs < 4; ++cs) {
    const bool ok = (cs < 2 ? hw : he) && ((cs == 0 || cs == 2) ? hs : hn);
    if (!ok) continue;
    const float tX = cs < 2 ? tw : te;
    const float tY = (cs == 0 || cs == 2) ? ts : tn;
    const float sY = (cs == 0 || cs == 2) ? -1.f : 1.f;
    const float U0 = t0x * tX;
    const float V0 = t0y * tX - sY * cy * (tX - tY);
    const float bx = K[(KF_BX + cs) * N + k], by = K[(KF_BY + cs) * N + k];
    const float A = K[(KF_A + cs) * N + k];
    const float CU = a * U0 - c * V0, CV = b * V0 - c * U0;
    const float C = U0 * CU + V0 * CV - f2;
    const float H = bx * U0 + by * V0;
    const float D = H * H - A * C;
    if (D >= 0.f) {
      const float ia = K[(KF_IA + cs) * N + k];
      const float s = sqrtf(D);
      const float d1 = (-H + s) * ia, d2 = (-H - s) * ia;
      const float x1 = bx * d1 + CU, y1 = by * d1 + CV;
      const float x2 = bx * d2 + CU, y2 = by * d2 + CV;
      const bool sx = cs < 2, sy = (cs == 0 || cs == 2);
      const bool c1 = (sx ? x1 >= 0.f : x1 <= 0.f) && (sy ? y1 >= 0.f : y1 <= 0.f);
      const bool c2 = (sx ? x2 >= 0.f : x2 <= 0.f) && (sy ? y2 >= 0.f : y2 <= 0.f);
      const float r1 = tX + d1, r2 = tX + d2;
      if (c1 && r1 < t) t = r1;
      if (c2 && r2 < t) t = r2;
    }
  }
  const float t0 = (float)T0d[k];
#pragma unroll
  for (int cs = 0; cs < 4; ++cs) {
    const bool ok = cs == 0 ? hw : cs == 1 ? he : cs == 2 ? hs : hn;
    if (!ok) continue;
    const float tnb = cs == 0 ? tw : cs == 1 ? te : cs == 2 ? ts : tn;
    const size_t nb = cs == 0 ? k - 1 : cs == 1 ? k + 1 : cs == 2 ? k - nx : k + nx;
    const float dis = cs < 2 ? K[KF_DX * N + k] : K[KF_DY * N + k];
    const float g = cs < 2 ? t0x : t0y;
    const float ip = K[(KF_IP + cs) * N + k];
    const float lim = tnb * (float)T0d[nb], half = tnb * 0.5f;
    const float r1 = tnb + (dis - g * tnb) * ip, r2 = tnb + (-dis - g * tnb) * ip;
    if (r1 * t0 >= lim && r1 > half && r1 < t) t = r1;
    if (r2 * t0 >= lim && r2 > half && r2 < t) t = r2;
  }
  return t;
}

__device__ inline void f32_sweeps(const PeriodDev& P, const F32Layout& L, SolveShared& sh) {
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  const Box box = sh.box;
  float* tau = L.tau;
  float* tau_old = L.tau_old;
  const float* K = L.K;
  const double* T0 = L.T0;
  int iter, status = ST_NOT_CONVERGED;
  for (iter = 1; iter <= MAXITER_UW; ++iter) {
    double l1 = 0.0, linf = 0.0;
    for (int s = 0; s < 4; ++s) {
      SweepGeom g;
      g.ilo = 0; g.ihi = nx - 1; g.jlo = 0; g.jhi = ny - 1;
      sweep_dirs(s, g.xdir, g.ydir);
      const int nd = g.ndiag();
      for (int d = 0; d < nd; ++d) {
        const int vlo = g.vmin(d), vhi = g.vmax(d);
        for (int v = vlo + (int)threadIdx.x; v <= vhi; v += blockDim.x) {
          int i, j;
          g.cell(d, v, i, j);
          if (box.has(i, j)) continue;
          const size_t k = (size_t)i + (size_t)nx * j;
          const float tb = tau[k];
          if (s == 0) tau_old[k] = tb;
          const float tn = f32_update(K, N, k, i, j, nx, ny, tau, T0, tb);
          tau[k] = tn;
          if (s == 3) {
            // FP64 convergence bookkeeping: exact difference of FP32 iterates
            const double dd = fabs((double)tn - (double)tau_old[k]) * T0[k];
            l1 += dd;
            linf = fmax(linf, dd);
          }
        }
        __syncthreads();
      }
    }
    block_sum_max(l1, linf, sh.red);
    l1 = l1 / (double)nx / (double)ny;
    if (fabs(l1) < TOL_UW && linf < TOL_UW) { status = ST_OK; break; }
  }
  if (threadIdx.x == 0) {
    sh.status = status;
    sh.iters = iter > MAXITER_UW ? MAXITER_UW : iter;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(128) k_batch_fp32(BatchArgs A) {
  __shared__ SolveShared sh;
  __shared__ int next;
  double* base = A.ws + (size_t)blockIdx.x * (size_t)A.ws_doubles;
  for (;;) {
    if (threadIdx.x == 0) next = atomicAdd(A.queue, 1);
    __syncthreads();
    const int q = next;
    __syncthreads();
    if (q >= A.nsolve) break;
    const int s = A.order[q];
    const PeriodDev P = A.periods[A.pidx[s]];
    const size_t N = (size_t)P.nx * P.ny;
    if (threadIdx.x == 0) sh.flag = ST_OK;
    F32Layout L = carve32(base, N);
    const double x0 = A.srcx[s] / 180.0 * PI_S, y0 = A.srcy[s] / 180.0 * PI_S;
    f32_setup(P, x0, y0, L, sh);
    if (sh.status != ST_OK) {
      const int st = sh.status;
      __syncthreads();
      // zero this solve's outputs
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
      if (threadIdx.x == 0) {
        A.chi[s] = 0.0;
        A.status[s] = st;
        A.fwd_iters[s] = 0;
        A.adj_iters[s] = 0;
        if (A.fwd_updates) A.fwd_updates[s] = 0;
      }
      __syncthreads();
      continue;
    }
    f32_sweeps(P, L, sh);
    const int fst = sh.status, fit = sh.iters;
    for (size_t k = threadIdx.x; k < N; k += blockDim.x) L.T[k] = (double)L.tau[k] * L.T0[k];
    if (A.fwd_updates && threadIdx.x == 0) {
      const Box b = sh.box;
      const double frozen = (double)(b.i1 - b.i0 + 1) * (b.j1 - b.j0 + 1);
      A.fwd_updates[s] = (double)fit * 4.0 * ((double)N - frozen);
    }
    __syncthreads();
    solve_tail(A, P, s, L.T, L.aw, sh, fst, fit);
  }
}

void launch_batch_fp32(const BatchArgs& a, int grid, int block, cudaStream_t st) {
  k_batch_fp32<<<grid, block, 0, st>>>(a);
}

int batch_fp32_max_blocks_per_sm(int block) {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_fp32, block, 0);
  return n;
}

}  // namespace sgb
