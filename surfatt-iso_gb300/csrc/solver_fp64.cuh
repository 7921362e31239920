// solver_fp64.cuh -- CTA-level FP64 building blocks of one (period, source)
// solve: factored first-order upwind eikonal (FSM_UW_PS_*), first-order
// adjoint (FSM_O1_JSE_*), WENO3 variants, mask, interp2, misfit.
//
// One thread block owns one solve.  Every routine is called by all threads of
// the block and ends with the block synchronised.  The sweeps walk
// anti-diagonals (SweepGeom) with one __syncthreads() per diagonal.
//
// Arithmetic: the plain path evaluates every per-cell quantity that the
// reference recomputes on each visit (px, py, eqn_a, the one-sided `dis`)
// exactly as the reference writes it, once per solve; on each visit it keeps
// the reference's formulas but with divisions by loop-invariant values
// turned into multiplications by stored reciprocals and the quadratic's
// coefficients grouped (eqn_b/2 = Bx*qx + By*qy, eqn_c = qx*Cx + qy*Cy - f^2).
// Results agree with the reference to rounding (relative 1e-12 level on
// converged travel times), not bit for bit.
#pragma once
#include "common.cuh"

namespace sgb {

// Per-cell constants of the plain forward sweep, one contiguous record of
// KC_COUNT doubles per cell (K[cell * KC_COUNT + index]): a visit reads one
// record instead of one word from each of 26 arrays.
enum FwdConst {
  KC_CX = 0,     // T0/dx
  KC_CY,         // T0/dy
  KC_PXM,        // T0x + T0/dx  (neighbour i-1)
  KC_PXP,        // T0x - T0/dx  (neighbour i+1)
  KC_PYM,        // T0y + T0/dy  (neighbour j-1)
  KC_PYP,        // T0y - T0/dy  (neighbour j+1)
  KC_EA,         // eqn_a of the four two-sided cases (4)
  KC_IEA = KC_EA + 4,   // 1/eqn_a (4)
  KC_BX = KC_IEA + 4,   // a*px - c*py (4)
  KC_BY = KC_BX + 4,    // b*py - c*px (4)
  KC_IPXM = KC_BY + 4,  // 1/pxm, 1/pxp, 1/pym, 1/pyp
  KC_IPXP,
  KC_IPYM,
  KC_IPYP,
  KC_COUNT
};

// Workspace of one forward solve (device pointers, N = nx*ny cells each).
struct FwdWs {
  double* tau;
  double* tau_old;
  double* T0;
  double* K;  // N records of KC_COUNT (hoisted path) or T0x, T0y arrays (WENO3)
};

// Frozen source box (:859-872): |(xx(i)-x0)/dx| <= R and |(yy(j)-y0)/dy| <= R.
// The test is separable; the box is [fi0, fi1] x [fj0, fj1] (empty if fi0 > fi1).
struct Box {
  int i0, i1, j0, j1;
  __device__ bool has(int i, int j) const { return i >= i0 && i <= i1 && j >= j0 && j <= j1; }
};

// Shared scratch a solve needs (static part of the block's shared memory).
struct SolveShared {
  double red[64];
  double fun0, x0, y0;
  int status;
  int iters;
  Box box;
  int flag;
};

// ---------------------------------------------------------------------------
// Forward setup: T0, its gradient, tau init and the hoisted constants.
// lon/lat: :801-872 (T0 = great-circle distance * fun0).  Cartesian UW:
// :47-90.  (x0, y0) in sweep units.  Returns status via sh.status.
// ---------------------------------------------------------------------------
// Work items (the batched kernel cutting a solve into items): `grad`, when
// given, holds the solve's T0 gradient (T0x at [k], T0y at [gstride + k]).
// resume = false: T0 and tau are initialised and the gradient stored there;
// resume = true: T0 (W.T0) and the gradient are read back, tau is left
// alone, and only the hoisted constants are rebuilt (to the same bits).
// part / nparts: this block sets up cells of the block-sized chunks
// part, part + nparts, ... (several blocks share one solve's setup).
__device__ inline void fwd_setup(const PeriodDev& P, double x0, double y0, double frozen_r,
                                 double tau_frozen, double tau_init, const FwdWs& W,
                                 bool hoist, SolveShared& sh, double* grad = nullptr,
                                 size_t gstride = 0, bool resume = false, int part = 0,
                                 int nparts = 1) {
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  if (threadIdx.x == 0) {
    sh.status = ST_OK;
    float r1 = 0.f, r2 = 0.f;
    int i0 = locate_cell(P.xs, nx - 1, P.dx, x0, &r1);
    int j0 = locate_cell(P.ys, ny - 1, P.dy, y0, &r2);
    if (i0 < 0 || j0 < 0) {
      sh.status = ST_BAD_ARG;
    } else {
      float w00 = (1 - r1) * (1 - r2), w01 = (1 - r1) * r2, w10 = r1 * (1 - r2), w11 = r1 * r2;
      size_t k00 = i0 + (size_t)nx * j0;
      sh.fun0 = (double)w00 * P.fun[k00] + (double)w01 * P.fun[k00 + nx] +
                (double)w10 * P.fun[k00 + 1] + (double)w11 * P.fun[k00 + nx + 1];
    }
    // frozen box, separable test
    int a0 = nx, a1 = -1, b0 = ny, b1 = -1;
    for (int i = 0; i < nx; ++i)
      if (fabs((P.xs[i] - x0) / P.dx) <= frozen_r) { a0 = min(a0, i); a1 = max(a1, i); }
    for (int j = 0; j < ny; ++j)
      if (fabs((P.ys[j] - y0) / P.dy) <= frozen_r) { b0 = min(b0, j); b1 = max(b1, j); }
    sh.box = Box{a0, a1, b0, b1};
    if (sh.status == ST_OK && a0 <= a1 && b0 <= b1 &&
        (a0 == 0 || a1 == nx - 1 || b0 == 0 || b1 == ny - 1))
      sh.status = ST_SOURCE_ON_BOUNDARY;
    sh.x0 = x0;
    sh.y0 = y0;
  }
  __syncthreads();
  if (sh.status != ST_OK) return;
  const double fun0 = sh.fun0;
  const Box box = sh.box;
  const double dx = P.dx, dy = P.dy;
  double cy0 = 0, sy0 = 0;
  if (P.lonlat) { cy0 = cos(y0); sy0 = sin(y0); }
  for (size_t k = threadIdx.x + (size_t)part * blockDim.x; k < N;
       k += (size_t)blockDim.x * nparts) {
    const int i = (int)(k % nx), j = (int)(k / nx);
    double t0, t0x, t0y;
    if (resume) {
      t0 = W.T0[k];
      t0x = grad[k];
      t0y = grad[gstride + k];
    } else if (P.lonlat) {
      const double cyy = P.cosy[j], syy = P.siny[j];
      const double cdx = cos(P.xs[i] - x0), sdx = sin(P.xs[i] - x0);
      const double tmp = syy * sy0 + cyy * cy0 * cdx;
      double cl = tmp < 1.0 ? tmp : 1.0;
      cl = cl > -1.0 ? cl : -1.0;
      t0 = acos(cl) * R_EARTH * fun0;
      if (t0 == 0) {
        t0x = 0; t0y = 0;
      } else {
        const double rs = 1.0 / sqrt(1 - tmp * tmp);
        t0x = -(rs * cyy * cy0 * (-1.0) * sdx * R_EARTH * fun0);
        t0y = -(rs * (cyy * sy0 - syy * cy0 * cdx) * R_EARTH * fun0);
      }
    } else {
      // Cartesian T0 with source-interpolated metric (:68-78); a0, b0, c0
      // are recomputed by every thread from the four source nodes.
      float r1 = 0.f, r2 = 0.f;
      int i0 = locate_cell(P.xs, nx - 1, dx, x0, &r1);
      int j0 = locate_cell(P.ys, ny - 1, dy, y0, &r2);
      float w00 = (1 - r1) * (1 - r2), w01 = (1 - r1) * r2, w10 = r1 * (1 - r2), w11 = r1 * r2;
      size_t k00 = i0 + (size_t)nx * j0;
      double a0 = (double)w00 * P.a[k00] + (double)w01 * P.a[k00 + nx] +
                  (double)w10 * P.a[k00 + 1] + (double)w11 * P.a[k00 + nx + 1];
      double b0 = (double)w00 * P.b[k00] + (double)w01 * P.b[k00 + nx] +
                  (double)w10 * P.b[k00 + 1] + (double)w11 * P.b[k00 + nx + 1];
      double c0 = (double)w00 * P.c[k00] + (double)w01 * P.c[k00 + nx] +
                  (double)w10 * P.c[k00 + 1] + (double)w11 * P.c[k00 + nx + 1];
      double D = a0 * b0 - c0 * c0;
      double ddx = P.xs[i] - x0, ddy = P.ys[j] - y0;
      t0 = fun0 * sqrt((b0 / D * (ddx * ddx) + a0 / D * (ddy * ddy) + 2 * c0 / D * ddx * ddy));
      if (t0 == 0) {
        t0x = 0; t0y = 0;
      } else {
        t0x = fun0 * fun0 * (b0 / D * ddx + c0 / D * ddy) / t0;
        t0y = fun0 * fun0 * (a0 / D * ddy + c0 / D * ddx) / t0;
      }
    }
    if (!resume) {
      W.T0[k] = t0;
      W.tau[k] = box.has(i, j) ? tau_frozen : tau_init;
      if (grad) {
        grad[k] = t0x;
        grad[gstride + k] = t0y;
      }
    }
    if (!hoist) {
      W.K[(size_t)0 * N + k] = t0x;
      W.K[(size_t)1 * N + k] = t0y;
      continue;
    }
    const double a = P.a[k], b = P.b[k], c = P.c[k];
    const double cx = t0 / dx, cy = t0 / dy;
    const double pxm = t0x + cx, pxp = t0x - cx, pym = t0y + cy, pyp = t0y - cy;
    double* K = W.K + k * (size_t)KC_COUNT;
    K[KC_CX] = cx;
    K[KC_CY] = cy;
    K[KC_PXM] = pxm;
    K[KC_PXP] = pxp;
    K[KC_PYM] = pym;
    K[KC_PYP] = pyp;
#pragma unroll
    for (int cs = 0; cs < 4; ++cs) {
      const double px = cs < 2 ? pxm : pxp;
      const double py = (cs == 0 || cs == 2) ? pym : pyp;
      const double ea = a * (px * px) + b * (py * py) - 2 * c * px * py;
      K[KC_EA + cs] = ea;
      K[KC_IEA + cs] = 1.0 / ea;
      K[KC_BX + cs] = a * px - c * py;
      K[KC_BY + cs] = b * py - c * px;
    }
    K[KC_IPXM] = 1.0 / pxm;
    K[KC_IPXP] = 1.0 / pxp;
    K[KC_IPYM] = 1.0 / pym;
    K[KC_IPYP] = 1.0 / pyp;
  }
  __syncthreads();
}

// Two-sided case cs of the plain first-order upwind update (:904-993):
// lowers t to each causal root of the case's quadratic.  q* are the scaled
// neighbour values (qw = -cx*tw, qe = cx*te, qs = -cy*ts, qn = cy*tn).
// (the case's constants ea, bx, by, 1/ea given: K[KC_EA + cs], ...)
__device__ __forceinline__ void uw_two_sided_v(int cs, double ea, double bx, double by,
                                               double iea, bool hw, bool he, bool hs, bool hn,
                                               double qw, double qe, double qs, double qn,
                                               double a, double b, double c, double f2,
                                               double& t) {
  const bool ok = (cs < 2 ? hw : he) && ((cs == 0 || cs == 2) ? hs : hn);
  if (!ok) return;
  const double qx = cs < 2 ? qw : qe;
  const double qy = (cs == 0 || cs == 2) ? qs : qn;
  const double Cx = a * qx - c * qy;
  const double Cy = b * qy - c * qx;
  const double ec = qx * Cx + qy * Cy - f2;
  const double hb = bx * qx + by * qy;
  const double del = hb * hb - ea * ec;
  if (del >= 0) {
    const double s = sqrt(del);
    const double r1 = (-hb + s) * iea, r2 = (-hb - s) * iea;
    const double x1 = bx * r1 + Cx, y1 = by * r1 + Cy;
    const double x2 = bx * r2 + Cx, y2 = by * r2 + Cy;
    const bool sx = cs < 2, sy = (cs == 0 || cs == 2);  // true: >= 0 required
    const bool c1 = (sx ? x1 >= 0 : x1 <= 0) && (sy ? y1 >= 0 : y1 <= 0);
    const bool c2 = (sx ? x2 >= 0 : x2 <= 0) && (sy ? y2 >= 0 : y2 <= 0);
    if (c1 && r1 < t) t = r1;
    if (c2 && r2 < t) t = r2;
  }
}

__device__ __forceinline__ void uw_two_sided(int cs, const double* __restrict__ K, bool hw,
                                             bool he, bool hs, bool hn, double qw, double qe,
                                             double qs, double qn, double a, double b, double c,
                                             double f2, double& t) {
  const bool ok = (cs < 2 ? hw : he) && ((cs == 0 || cs == 2) ? hs : hn);
  if (!ok) return;
  uw_two_sided_v(cs, K[KC_EA + cs], K[KC_BX + cs], K[KC_BY + cs], K[KC_IEA + cs], hw, he, hs, hn,
                 qw, qe, qs, qn, a, b, c, f2, t);
}

// Neighbour of cell k across face cs (0 west, 1 east, 2 south, 3 north).
__device__ __forceinline__ size_t uw_nb(int cs, size_t k, int nx) {
  return cs == 0 ? k - 1 : cs == 1 ? k + 1 : cs == 2 ? k - nx : k + nx;
}

// One-sided case cs (0 west, 1 east, 2 south, 3 north) of the same update
// (:996-1075): lowers t to each admissible root along one axis.  (ip =
// K[KC_IPXM + cs], t0nb = T0 of the neighbour across face cs, dis = disx for
// cs < 2 and disy otherwise.)
__device__ __forceinline__ void uw_one_sided_v(int cs, double ip, double t0nb, double dis,
                                               bool hw, bool he, bool hs, bool hn, double qw,
                                               double qe, double qs, double qn, double tw,
                                               double te, double ts, double tn, double t0,
                                               double& t) {
  const bool ok = cs == 0 ? hw : cs == 1 ? he : cs == 2 ? hs : hn;
  if (!ok) return;
  const double q = cs == 0 ? qw : cs == 1 ? qe : cs == 2 ? qs : qn;
  const double tnb = cs == 0 ? tw : cs == 1 ? te : cs == 2 ? ts : tn;
  const double lim = tnb * t0nb, half = tnb * 0.5;
  const double r1 = (dis - q) * ip, r2 = (-dis - q) * ip;
  if (r1 * t0 >= lim && r1 > half && r1 < t) t = r1;
  if (r2 * t0 >= lim && r2 > half && r2 < t) t = r2;
}

__device__ __forceinline__ void uw_one_sided(int cs, const double* __restrict__ K, size_t k,
                                             int nx, const double* __restrict__ T0, bool hw,
                                             bool he, bool hs, bool hn, double qw, double qe,
                                             double qs, double qn, double tw, double te,
                                             double ts, double tn, double disx, double disy,
                                             double t0, double& t) {
  const bool ok = cs == 0 ? hw : cs == 1 ? he : cs == 2 ? hs : hn;
  if (!ok) return;
  uw_one_sided_v(cs, K[KC_IPXM + cs], T0[uw_nb(cs, k, nx)], cs < 2 ? disx : disy, hw, he, hs, hn,
                 qw, qe, qs, qn, tw, te, ts, tn, t0, t);
}

// One visit of cell k by the plain first-order upwind update (:904-1079):
// returns min(tau, every causal two-sided root, every admissible one-sided
// root).  `tau` may be global or shared memory (same layout).
__device__ __forceinline__ double uw_update(const double* __restrict__ Kall, size_t N, size_t k,
                                            int i, int j, int nx, int ny,
                                            const double* __restrict__ tau,
                                            const double* __restrict__ T0, double a, double b,
                                            double c, double f2, double disx, double disy,
                                            double t) {
  const bool hw = i > 0, he = i < nx - 1, hs = j > 0, hn = j < ny - 1;
  const double* __restrict__ K = Kall + k * (size_t)KC_COUNT;
  const double cx = K[KC_CX], cy = K[KC_CY];
  const double tw = hw ? tau[k - 1] : 0.0, te = he ? tau[k + 1] : 0.0;
  const double ts = hs ? tau[k - nx] : 0.0, tn = hn ? tau[k + nx] : 0.0;
  const double qw = -(cx * tw), qe = cx * te, qs = -(cy * ts), qn = cy * tn;
#pragma unroll
  for (int cs = 0; cs < 4; ++cs) uw_two_sided(cs, K, hw, he, hs, hn, qw, qe, qs, qn, a, b, c, f2, t);
  const double t0 = T0[k];
#pragma unroll
  for (int cs = 0; cs < 4; ++cs)
    uw_one_sided(cs, K, k, nx, T0, hw, he, hs, hn, qw, qe, qs, qn, tw, te, ts, tn, disx, disy, t0,
                 t);
  return t;
}

// The candidates of one case only (two-sided case cs and one-sided case cs):
// their minimum, +inf when the case has none.  The minimum over the four
// cases and the old value is uw_update's result.
__device__ __forceinline__ double uw_case(int cs, const double* __restrict__ Kall, size_t k, int i,
                                          int j, int nx, int ny, const double* __restrict__ tau,
                                          const double* __restrict__ T0, double a, double b,
                                          double c, double f2, double disx, double disy) {
  const bool hw = i > 0, he = i < nx - 1, hs = j > 0, hn = j < ny - 1;
  const double* __restrict__ K = Kall + k * (size_t)KC_COUNT;
  const double cx = K[KC_CX], cy = K[KC_CY];
  const double tw = hw ? tau[k - 1] : 0.0, te = he ? tau[k + 1] : 0.0;
  const double ts = hs ? tau[k - nx] : 0.0, tn = hn ? tau[k + nx] : 0.0;
  const double qw = -(cx * tw), qe = cx * te, qs = -(cy * ts), qn = cy * tn;
  double t = __longlong_as_double(0x7ff0000000000000LL);
  uw_two_sided(cs, K, hw, he, hs, hn, qw, qe, qs, qn, a, b, c, f2, t);
  uw_one_sided(cs, K, k, nx, T0, hw, he, hs, hn, qw, qe, qs, qn, tw, te, ts, tn, disx, disy, T0[k],
               t);
  return t;
}

// Forward sweeps until |dtau|*T0 is below tol in L1 (mean) and Linf
// (:881-1122).  tau_old is captured on each cell's first visit of an
// iteration and the change is accumulated on its last visit.
// Iterations it0 .. max_iter: sh.status = ST_OK and sh.iters = the
// iteration that converged, or ST_NOT_CONVERGED and max_iter.
__device__ inline void uw_sweeps(const PeriodDev& P, const FwdWs& W, SolveShared& sh,
                                 int max_iter, int it0 = 1) {
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  const Box box = sh.box;
  double* __restrict__ tau = W.tau;
  double* __restrict__ tau_old = W.tau_old;
  const double* __restrict__ K = W.K;
  const double* __restrict__ T0 = W.T0;
  int iter;
  int status = ST_NOT_CONVERGED;
  for (iter = it0; iter <= max_iter; ++iter) {
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
          const double tb = tau[k];
          if (s == 0) tau_old[k] = tb;
          const double tn = uw_update(K, N, k, i, j, nx, ny, tau, T0, P.a[k], P.b[k], P.c[k],
                                      P.f2[k], P.disx[k], P.disy[k], tb);
          tau[k] = tn;
          if (s == 3) {
            const double dd = fabs(tn - tau_old[k]) * T0[k];
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
    sh.iters = iter > max_iter ? max_iter : iter;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Adjoint (FSM_O1_JSE_*): coefficients (:1348-1370), sweeps (:1382-1443).
// Up to two right-hand sides share the coefficients (measadj.f90:85 and :99
// call the solver twice with the same travel-time field); each field keeps
// its own convergence test and stops exactly when the reference's separate
// call would.
// ---------------------------------------------------------------------------
enum AdjConst { KA_WW = 0, KA_WE, KA_WS, KA_WN, KA_ID, KA_COUNT };

struct AdjWs {
  const double* T;     // travel times (N)
  double* K;           // KA_COUNT * N
  double* delta[2];    // right-hand sides (N)
  double* Ta[2];       // fields (N)
  double* old[2];      // snapshots (N)
};

// Coefficients: Ta = (delta + e)/d with e = (Ta_W*a1p - Ta_E*a2m)/dx
// + (Ta_S*b1p - Ta_N*b2m)/dy is stored as weights w* = coef/(h*d) and 1/d;
// |d| < eps gives Ta = 0 (:1394-1395) through zero weights and 1/d = 0.
__device__ inline void adj_setup(const PeriodDev& P, const AdjWs& W, int nfield) {
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  const double dx = P.dx, dy = P.dy;
  const double* T = W.T;
  const double *a = P.a, *b = P.b, *c = P.c;
  for (size_t k = threadIdx.x; k < N; k += blockDim.x) {
    const int i = (int)(k % nx), j = (int)(k / nx);
    const bool interior = i > 0 && i < nx - 1 && j > 0 && j < ny - 1;
    if (!interior) {
      for (int f = 0; f < nfield; ++f) W.Ta[f][k] = 0.0;
      continue;
    }
    const size_t w = k - 1, e = k + 1, s = k - nx, n = k + nx;
    const double a1 = -((T[k] - T[w]) / dx * (a[k] + a[w]) / 2) +
                      (T[n] - T[s] + T[w + nx] - T[w - nx]) / (4 * dy) * (c[k] + c[w]) / 2;
    const double a2 = -((T[e] - T[k]) / dx * (a[e] + a[k]) / 2) +
                      (T[e + nx] - T[e - nx] + T[n] - T[s]) / (4 * dy) * (c[e] + c[k]) / 2;
    const double b1 = -((T[k] - T[s]) / dy * (b[k] + b[s]) / 2) +
                      (T[e] - T[w] + T[s + 1] - T[s - 1]) / (4 * dx) * (c[k] + c[s]) / 2;
    const double b2 = -((T[n] - T[k]) / dy * (b[n] + b[k]) / 2) +
                      (T[n + 1] - T[n - 1] + T[e] - T[w]) / (4 * dx) * (c[n] + c[k]) / 2;
    const double a1m = (a1 - fabs(a1)) / 2, a1p = (a1 + fabs(a1)) / 2;
    const double a2m = (a2 - fabs(a2)) / 2, a2p = (a2 + fabs(a2)) / 2;
    const double b1m = (b1 - fabs(b1)) / 2, b1p = (b1 + fabs(b1)) / 2;
    const double b2m = (b2 - fabs(b2)) / 2, b2p = (b2 + fabs(b2)) / 2;
    const double d = (a2p - a1m) / dx + (b2p - b1m) / dy;
    double id = 0, ww = 0, we = 0, ws = 0, wn = 0;
    if (!(fabs(d) < EPS14)) {
      id = 1.0 / d;
      ww = a1p / dx * id;
      we = -(a2m / dx) * id;
      ws = b1p / dy * id;
      wn = -(b2m / dy) * id;
    }
    double* Kr = W.K + k * (size_t)KA_COUNT;  // one record per cell
    Kr[KA_WW] = ww;
    Kr[KA_WE] = we;
    Kr[KA_WS] = ws;
    Kr[KA_WN] = wn;
    Kr[KA_ID] = id;
    for (int f = 0; f < nfield; ++f) W.Ta[f][k] = 100;
  }
  __syncthreads();
}

// returns iterations of field f in its[f]; statuses in st[f]
__device__ inline void adj_sweeps(const PeriodDev& P, const AdjWs& W, int nfield, SolveShared& sh,
                                  int* its, int* sts) {
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  const double* __restrict__ K = W.K;
  bool active[2] = {nfield > 0, nfield > 1};
  int iters[2] = {MAXITER_JSE, MAXITER_JSE};
  int stat[2] = {ST_NOT_CONVERGED, ST_NOT_CONVERGED};
  for (int iter = 1; iter <= MAXITER_JSE && (active[0] || active[1]); ++iter) {
    double l1[2] = {0, 0}, lm[2] = {0, 0};
    for (int s = 0; s < 4; ++s) {
      SweepGeom g;
      g.ilo = 1; g.ihi = nx - 2; g.jlo = 1; g.jhi = ny - 2;
      sweep_dirs(s, g.xdir, g.ydir);
      const int nd = g.ndiag();
      for (int d = 0; d < nd; ++d) {
        const int vlo = g.vmin(d), vhi = g.vmax(d);
        for (int v = vlo + (int)threadIdx.x; v <= vhi; v += blockDim.x) {
          int i, j;
          g.cell(d, v, i, j);
          const size_t k = (size_t)i + (size_t)nx * j;
          const double* Kr = K + k * (size_t)KA_COUNT;
          const double ww = Kr[KA_WW], we = Kr[KA_WE];
          const double ws = Kr[KA_WS], wn = Kr[KA_WN];
          const double id = Kr[KA_ID];
#pragma unroll
          for (int f = 0; f < 2; ++f) {
            if (!active[f]) continue;
            double* __restrict__ ta = W.Ta[f];
            const double before = ta[k];
            if (s == 0) W.old[f][k] = before;
            const double nv = W.delta[f][k] * id + ww * ta[k - 1] + we * ta[k + 1] +
                              ws * ta[k - nx] + wn * ta[k + nx];
            ta[k] = nv;
            if (s == 3) {
              const double dd = fabs(nv - W.old[f][k]);
              l1[f] += dd;
              lm[f] = fmax(lm[f], dd);
            }
          }
        }
        __syncthreads();
      }
    }
    for (int f = 0; f < 2; ++f) {
      if (!active[f]) continue;
      double s1 = l1[f], sm = lm[f];
      block_sum_max(s1, sm, sh.red);
      s1 = s1 / (double)(nx * ny);
      if (fabs(s1) < TOL_JSE && sm < TOL_JSE) {
        active[f] = false;
        iters[f] = iter;
        stat[f] = ST_OK;
      }
    }
  }
  for (int f = 0; f < nfield; ++f) {
    its[f] = iters[f];
    sts[f] = stat[f];
  }
}

// Bilinear splat of adjoint sources (:1328-1336) by one thread, in receiver
// order (the reference's accumulation order).  lon/lat scales by the cell
// area dx*R*cos(lat_rec)*dy*R, Cartesian by dx*dy.  Returns ST_BAD_ARG for a
// receiver outside the grid.
__device__ inline int adj_splat(const PeriodDev& P, double* delta, int nrec, const double* recx,
                                const double* recy, const double* sadj, double sadj_scale) {
  const int nx = P.nx, ny = P.ny;
  for (int r = 0; r < nrec; ++r) {
    double xr = recx[r], yr = recy[r];
    if (P.lonlat) {
      xr = xr / 180.0 * PI_S;
      yr = yr / 180.0 * PI_S;
    }
    float r1 = 0.f, r2 = 0.f;
    const int i0 = locate_cell(P.xs, nx, P.dx, xr, &r1);
    const int j0 = locate_cell(P.ys, ny, P.dy, yr, &r2);
    if (i0 < 0 || j0 < 0) return ST_BAD_ARG;
    const double den = P.lonlat ? P.dx * R_EARTH * cos(yr) * P.dy * R_EARTH : P.dx * P.dy;
    const double s = sadj ? sadj[r] : sadj_scale;
    const size_t k = i0 + (size_t)nx * j0;
    delta[k] += s * (double)(1 - r1) * (double)(1 - r2) / den;
    if (j0 + 1 < ny) delta[k + nx] += s * (double)(1 - r1) * (double)r2 / den;
    if (i0 + 1 < nx) delta[k + 1] += s * (double)r1 * (double)(1 - r2) / den;
    if (i0 + 1 < nx && j0 + 1 < ny) delta[k + nx + 1] += s * (double)r1 * (double)r2 / den;
  }
  return ST_OK;
}

// interp2_0_dp (src/shared/utils.f90:917-942) on increasing coordinates:
// x1 = last node <= xq, x2 = x1+1.  Returns false outside the grid.
__device__ inline bool interp2(const double* x, int nx, const double* y, int ny, const double* v,
                               double xq, double yq, double* out) {
  int lo = -1, hi = nx;  // x[lo] <= xq < x[hi]
  while (hi - lo > 1) {
    int m = (lo + hi) >> 1;
    if (xq >= x[m]) lo = m; else hi = m;
  }
  if (lo < 0 || lo >= nx - 1) return false;
  int ylo = -1, yhi = ny;
  while (yhi - ylo > 1) {
    int m = (ylo + yhi) >> 1;
    if (yq >= y[m]) ylo = m; else yhi = m;
  }
  if (ylo < 0 || ylo >= ny - 1) return false;
  const int x1 = lo, x2 = lo + 1, y1 = ylo, y2 = ylo + 1;
  const double vn = fabs((x[x2] - x[x1]) * (y[y2] - y[y1]));
  const double n1 = fabs((x[x2] - xq) * (y[y2] - yq));
  const double n2 = fabs((x[x1] - xq) * (y[y2] - yq));
  const double n3 = fabs((x[x2] - xq) * (y[y1] - yq));
  const double n4 = fabs((x[x1] - xq) * (y[y1] - yq));
  double r = 0;
  r = r + v[x1 + (size_t)nx * y1] * (n1 / vn);
  r = r + v[x2 + (size_t)nx * y1] * (n2 / vn);
  r = r + v[x1 + (size_t)nx * y2] * (n3 / vn);
  r = r + v[x2 + (size_t)nx * y2] * (n4 / vn);
  *out = r;
  return true;
}

// mask (:1449-1467): zero |xx-x0| < 1.5 dx and |yy-y0| < 1.5 dy (caller units).
__device__ inline void apply_mask(const PeriodDev& P, double* tab, double x0, double y0) {
  const int nx = P.nx, ny = P.ny;
  const double dx = P.xdeg[1] - P.xdeg[0], dy = P.ydeg[1] - P.ydeg[0];
  const size_t N = (size_t)nx * ny;
  for (size_t k = threadIdx.x; k < N; k += blockDim.x) {
    const int i = (int)(k % nx), j = (int)(k / nx);
    if (fabs(P.xdeg[i] - x0) < 1.5 * dx && fabs(P.ydeg[j] - y0) < 1.5 * dy) tab[k] = 0;
  }
  __syncthreads();
}

}  // namespace sgb
