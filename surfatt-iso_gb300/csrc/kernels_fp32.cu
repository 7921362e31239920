// kernels_fp32.cu -- the batched solve with the factored unknown tau = T/T0
// swept in FP32.
//
// What stays FP64: the analytic spherical T0 and its gradient (computed in
// FP64 per solve, then rounded once to FP32 for the sweep), the convergence
// decisions (sums and maxima of exact FP64 differences of the FP32 iterates),
// the travel times T = tau*T0, receiver interpolation, misfit, adjoint
// sources, and the kernel slots and their per-period sums.
//
// The FP32 forward sweep does not evaluate the reference's quadratic in tau
// directly: with tau = tau_X + delta (tau_X the case's x neighbour) the terms
// px*tau + qx = T0x*tau_X + px*delta and
// py*tau + qy = T0y*tau_X - sY*cy*(tau_X - tau_Y) + py*delta carry no
// cancellation between the O(T0/dx) terms, so delta (and tau) keep FP32
// relative accuracy.  It is the same local equation and the same candidate
// set (causal two-sided roots, admissible one-sided roots, min) as
// FSM_UW_PS_lonlat_2d (src/eikon_solver_2d.f90:904-1079).
//
// The adjoint is swept in FP32 too (coefficients from FP64 travel-time
// differences, :1348-1370); it stops at the reference's absolute tolerance
// or when the largest change falls to the FP32 resolution of the field.
//
// Layout: tau (and then each adjoint field) lives in shared memory with an
// even row pitch, so the cells of an anti-diagonal (address stride pitch-1 or
// pitch+1, both odd) hit distinct banks.  Each thread owns one cell of every
// diagonal; its operands for the next diagonal are loaded into registers
// before the current diagonal is computed, so the global/L2 latency overlaps
// the compute and the barrier.  Grids too large for shared memory keep tau in
// global memory (same code, other instantiation).
#include "kernels.cuh"
#include "solver_fp64.cuh"
#include "batch_tail.cuh"

namespace sgb {

constexpr int F32_MAX_THREADS = 512;        // longest anti-diagonal supported
constexpr size_t F32_SMEM_CAP = 110 * 1024;  // tau in shared memory up to this size

__host__ __device__ inline int f32_pitch(int nx) { return nx + (nx & 1); }

// Workspace per slot, in doubles: T0 and T (FP64), two adjoint right-hand
// sides (FP64), then FP32 arrays T0, T0x, T0y, old, 4 adjoint weights, two
// scaled sources and the global-memory tau (pitched).
long long batch_fp32_ws_doubles(long long N) {
  const long long f64 = 4 * N;
  const long long f32 = 11 * N + (N + 2 * 4096);  // pitched tau: (nx+1)*ny <= N + ny
  return f64 + (f32 + 1) / 2 + 64;
}

size_t batch_fp32_smem_bytes(long long max_pitched_cells, int max_nx, int* tau_resident) {
  const size_t cols = (size_t)max_nx * 16;
  const size_t tau = (size_t)max_pitched_cells * 4;
  *tau_resident = cols + tau <= F32_SMEM_CAP;
  return *tau_resident ? cols + tau : cols;
}

int batch_fp32_pitch(int nx) { return f32_pitch(nx); }

struct F32View {
  double* T0d;
  double* T;
  double* delta[2];
  float* T0f;
  float* gx;
  float* gy;
  float* old;
  float* W;       // 4N: ww, we, ws, wn
  float* src[2];  // delta*(1/d) per field
  float* gtau;
};

__device__ inline F32View carve32(double* base, size_t N) {
  F32View V;
  V.T0d = base;
  V.T = base + N;
  V.delta[0] = base + 2 * N;
  V.delta[1] = base + 3 * N;
  float* f = reinterpret_cast<float*>(base + 4 * N);
  V.T0f = f;
  V.gx = f + N;
  V.gy = f + 2 * N;
  V.old = f + 3 * N;
  V.W = f + 4 * N;
  V.src[0] = f + 8 * N;
  V.src[1] = f + 9 * N;
  V.gtau = f + 10 * N;
  return V;
}

// ---------------------------------------------------------------------------
// Setup: source slowness, frozen box, FP64 T0 and gradient (:828-872).
// cos/sin(x - x0) depend on the column only and are computed once per column.
// ---------------------------------------------------------------------------
__device__ inline void f32_setup(const PeriodDev& P, double x0, double y0, const F32View& V,
                                 float* tau, int pitch, double* colc, double* cols,
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
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    colc[i] = cos(P.xs[i] - x0);
    cols[i] = sin(P.xs[i] - x0);
  }
  __syncthreads();
  if (sh.status != ST_OK) return;
  const double fun0 = sh.fun0;
  const Box box = sh.box;
  const double cy0 = cos(y0), sy0 = sin(y0);
  for (size_t k = threadIdx.x; k < N; k += blockDim.x) {
    const int i = (int)(k % nx), j = (int)(k / nx);
    const double cyy = P.cosy[j], syy = P.siny[j];
    const double tmp = syy * sy0 + cyy * cy0 * colc[i];
    double cl = tmp < 1.0 ? tmp : 1.0;
    cl = cl > -1.0 ? cl : -1.0;
    const double t0 = acos(cl) * R_EARTH * fun0;
    double t0x = 0, t0y = 0;
    if (t0 != 0) {
      const double rs = rsqrt(1 - tmp * tmp) * R_EARTH * fun0;
      t0x = rs * cyy * cy0 * cols[i];
      t0y = -(rs * (cyy * sy0 - syy * cy0 * colc[i]));
    }
    V.T0d[k] = t0;
    V.T0f[k] = (float)t0;
    V.gx[k] = (float)t0x;
    V.gy[k] = (float)t0y;
    tau[i + (size_t)pitch * j] = box.has(i, j) ? 1.0f : 10.0f;
  }
  __syncthreads();
}

// Operands of one forward visit, loaded one diagonal ahead.
struct FwdOps {
  int k, t;          // cell index (x fastest), pitched index
  short i, j;
  bool on;
  float t0, gx, gy, a, b, c, f2, dsx, dsy, t0w, t0e, t0s, t0n, old;
  double t0d;
};

__device__ __forceinline__ void fwd_load(FwdOps& o, const SweepGeom& g, int d, int nd,
                                         const PeriodDev& P, const F32View& V, const Box& box,
                                         int pitch, bool last_sweep) {
  o.on = false;
  if (d >= nd) return;
  const int v = g.vmin(d) + (int)threadIdx.x;
  if (v > g.vmax(d)) return;
  int i, j;
  g.cell(d, v, i, j);
  if (box.has(i, j)) return;
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  const int k = i + nx * j;
  o.on = true;
  o.k = k;
  o.t = i + pitch * j;
  o.i = (short)i;
  o.j = (short)j;
  o.t0 = V.T0f[k];
  o.gx = V.gx[k];
  o.gy = V.gy[k];
  const float* F = P.f32;
  o.a = F[k];
  o.b = F[N + k];
  o.c = F[2 * N + k];
  o.f2 = F[3 * N + k];
  o.dsx = F[4 * N + k];
  o.dsy = F[5 * N + k];
  o.t0w = i > 0 ? V.T0f[k - 1] : 0.f;
  o.t0e = i < nx - 1 ? V.T0f[k + 1] : 0.f;
  o.t0s = j > 0 ? V.T0f[k - nx] : 0.f;
  o.t0n = j < ny - 1 ? V.T0f[k + nx] : 0.f;
  if (last_sweep) {
    o.old = V.old[k];
    o.t0d = V.T0d[k];
  }
}

// Packed FP32x2 helpers (one instruction for two lanes of a pair of cases).
__device__ __forceinline__ float2 bc2(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// Candidate of a two-sided root that passes the case's causality test
// (characteristic signs sx, sy: +1 requires >= 0, -1 requires <= 0).
__device__ __forceinline__ float causal_pick(float r, float chx, float chy, float sx, float sy,
                                             bool ok) {
  const bool cx = sx > 0.f ? chx >= 0.f : chx <= 0.f;
  const bool cy = sy > 0.f ? chy >= 0.f : chy <= 0.f;
  return (ok && cx && cy) ? r : __int_as_float(0x7f800000);
}

// Two two-sided cases sharing the y neighbour (tY, py, sY): lane .x uses the
// west neighbour (px = T0x + cx), lane .y the east one (px = T0x - cx).
// Returns the smaller admissible root of the two cases (or +inf).
__device__ __forceinline__ float two_sided_pair(float2 px, float2 tX, float2 U0, float py,
                                                float tY, float sY, float gy, float cy, float a,
                                                float b, float c, float f2, bool okx, bool oky) {
  const float2 A = fma2(px, fma2(bc2(a), px, bc2(-2.f * c * py)), bc2(b * py * py));
  const float2 bx = fma2(bc2(a), px, bc2(-c * py));
  const float2 by = fma2(bc2(-c), px, bc2(b * py));
  const float2 V0 = fma2(bc2(gy), tX, mul2(bc2(-sY * cy), add2(tX, bc2(-tY))));
  const float2 CU = fma2(bc2(a), U0, mul2(bc2(-c), V0));
  const float2 CV = fma2(bc2(b), V0, mul2(bc2(-c), U0));
  const float2 C = fma2(U0, CU, fma2(V0, CV, bc2(-f2)));
  const float2 H = fma2(bx, U0, mul2(by, V0));
  const float2 D = fma2(H, H, mul2(neg2(A), C));
  const bool vx = okx && D.x >= 0.f, vy = oky && D.y >= 0.f;
  const float2 sq = make_float2(fsqrt_fast(D.x), fsqrt_fast(D.y));
  const float2 ia = make_float2(frcp_fast(A.x), frcp_fast(A.y));
  const float2 d1 = mul2(add2(sq, neg2(H)), ia);
  const float2 d2 = mul2(add2(neg2(sq), neg2(H)), ia);
  const float2 x1 = fma2(bx, d1, CU), y1 = fma2(by, d1, CV);
  const float2 x2 = fma2(bx, d2, CU), y2 = fma2(by, d2, CV);
  const float2 r1 = add2(tX, d1), r2 = add2(tX, d2);
  const float sy = -sY;  // y neighbour j-1 (sY = -1) requires chy >= 0
  float m = causal_pick(r1.x, x1.x, y1.x, 1.f, sy, vx);
  m = fminf(m, causal_pick(r2.x, x2.x, y2.x, 1.f, sy, vx));
  m = fminf(m, causal_pick(r1.y, x1.y, y1.y, -1.f, sy, vy));
  m = fminf(m, causal_pick(r2.y, x2.y, y2.y, -1.f, sy, vy));
  return m;
}

// Two one-sided cases (lanes x, y): tau = tnb + (+-dis - g*tnb)/p, admitted
// when tau*T0 >= tnb*T0nb and tau > tnb/2 (:1017-1028).
__device__ __forceinline__ float one_sided_pair(float2 p, float2 tnb, float2 t0nb, float g,
                                                float dis, float t0, bool okx, bool oky) {
  const float2 ip = make_float2(frcp_fast(p.x), frcp_fast(p.y));
  const float2 gt = mul2(bc2(g), tnb);
  const float2 r1 = fma2(add2(bc2(dis), neg2(gt)), ip, tnb);
  const float2 r2 = fma2(add2(bc2(-dis), neg2(gt)), ip, tnb);
  const float2 lim = mul2(tnb, t0nb), half = mul2(tnb, bc2(0.5f));
  const float2 s1 = mul2(r1, bc2(t0)), s2 = mul2(r2, bc2(t0));
  const float inf = __int_as_float(0x7f800000);
  float m = (okx && s1.x >= lim.x && r1.x > half.x) ? r1.x : inf;
  m = fminf(m, (okx && s2.x >= lim.x && r2.x > half.x) ? r2.x : inf);
  m = fminf(m, (oky && s1.y >= lim.y && r1.y > half.y) ? r1.y : inf);
  m = fminf(m, (oky && s2.y >= lim.y && r2.y > half.y) ? r2.y : inf);
  return m;
}

// One FP32 visit (tau = tau_X + delta form); returns the new tau.
__device__ __forceinline__ float fwd_visit(const FwdOps& o, const float* tau, int pitch, int nx,
                                           int ny, float idx, float idy) {
  const int i = o.i, j = o.j, t = o.t;
  const bool hw = i > 0, he = i < nx - 1, hs = j > 0, hn = j < ny - 1;
  const float cur = tau[t];
  const float tw = hw ? tau[t - 1] : 0.f, te = he ? tau[t + 1] : 0.f;
  const float ts = hs ? tau[t - pitch] : 0.f, tn = hn ? tau[t + pitch] : 0.f;
  const float cx = o.t0 * idx, cy = o.t0 * idy;
  const float2 px = make_float2(o.gx + cx, o.gx - cx);
  const float2 tX = make_float2(tw, te);
  const float2 U0 = mul2(bc2(o.gx), tX);
  // (W,S), (E,S): y neighbour j-1, py = T0y + cy (:913-930)
  float m = two_sided_pair(px, tX, U0, o.gy + cy, ts, -1.f, o.gy, cy, o.a, o.b, o.c, o.f2,
                           hw && hs, he && hs);
  // (W,N), (E,N): y neighbour j+1, py = T0y - cy
  m = fminf(m, two_sided_pair(px, tX, U0, o.gy - cy, tn, 1.f, o.gy, cy, o.a, o.b, o.c, o.f2,
                              hw && hn, he && hn));
  // one-sided along x (W, E) and along y (S, N) (:996-1075)
  m = fminf(m, one_sided_pair(px, tX, make_float2(o.t0w, o.t0e), o.gx, o.dsx, o.t0, hw, he));
  m = fminf(m, one_sided_pair(make_float2(o.gy + cy, o.gy - cy), make_float2(ts, tn),
                              make_float2(o.t0s, o.t0n), o.gy, o.dsy, o.t0, hs, hn));
  return fminf(cur, m);
}

__device__ inline void f32_fwd_sweeps(const PeriodDev& P, const F32View& V, float* tau, int pitch,
                                      SolveShared& sh) {
  const int nx = P.nx, ny = P.ny;
  const Box box = sh.box;
  const float idx = (float)(1.0 / P.dx), idy = (float)(1.0 / P.dy);
  int iter, status = ST_NOT_CONVERGED;
  for (iter = 1; iter <= MAXITER_UW; ++iter) {
    double l1 = 0.0, linf = 0.0;
    for (int s = 0; s < 4; ++s) {
      SweepGeom g;
      g.ilo = 0; g.ihi = nx - 1; g.jlo = 0; g.jhi = ny - 1;
      sweep_dirs(s, g.xdir, g.ydir);
      const int nd = g.ndiag();
      FwdOps cur, nxt;
      fwd_load(cur, g, 0, nd, P, V, box, pitch, s == 3);
      for (int d = 0; d < nd; ++d) {
        fwd_load(nxt, g, d + 1, nd, P, V, box, pitch, s == 3);
        if (cur.on) {
          const float tb = tau[cur.t];
          const float tn = fwd_visit(cur, tau, pitch, nx, ny, idx, idy);
          tau[cur.t] = tn;
          if (s == 0) V.old[cur.k] = tb;
          if (s == 3) {
            const double dd = fabs((double)tn - (double)cur.old) * cur.t0d;
            l1 += dd;
            linf = fmax(linf, dd);
          }
        }
        __syncthreads();
        cur = nxt;
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

// ---------------------------------------------------------------------------
// FP32 adjoint
// ---------------------------------------------------------------------------
// Weights of Ta = src + ww*Ta_W + we*Ta_E + ws*Ta_S + wn*Ta_N from the face
// fluxes of :1348-1370 (travel-time differences in FP64, the rest FP32), and
// the scaled sources src_f = delta_f / d.
__device__ inline void f32_adj_setup(const PeriodDev& P, const F32View& V, int nf) {
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  const double* T = V.T;
  const float* F = P.f32;
  const float idx = (float)(1.0 / P.dx), idy = (float)(1.0 / P.dy);
  for (size_t k = threadIdx.x; k < N; k += blockDim.x) {
    const int i = (int)(k % nx), j = (int)(k / nx);
    if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1) continue;
    const size_t w = k - 1, e = k + 1, s = k - nx, n = k + nx;
    const float ak = F[k], aw = F[w], ae = F[e];
    const float bk = F[N + k], bs = F[N + s], bn = F[N + n];
    const float ck = F[2 * N + k], cw = F[2 * N + w], ce = F[2 * N + e], cs = F[2 * N + s],
                cn = F[2 * N + n];
    const float dkw = (float)(T[k] - T[w]), dek = (float)(T[e] - T[k]);
    const float dks = (float)(T[k] - T[s]), dnk = (float)(T[n] - T[k]);
    const float ya1 = (float)(T[n] - T[s] + T[w + nx] - T[w - nx]);
    const float ya2 = (float)(T[e + nx] - T[e - nx] + T[n] - T[s]);
    const float xb1 = (float)(T[e] - T[w] + T[s + 1] - T[s - 1]);
    const float xb2 = (float)(T[n + 1] - T[n - 1] + T[e] - T[w]);
    const float a1 = -(dkw * idx * (ak + aw) * 0.5f) + ya1 * (0.25f * idy) * (ck + cw) * 0.5f;
    const float a2 = -(dek * idx * (ae + ak) * 0.5f) + ya2 * (0.25f * idy) * (ce + ck) * 0.5f;
    const float b1 = -(dks * idy * (bk + bs) * 0.5f) + xb1 * (0.25f * idx) * (ck + cs) * 0.5f;
    const float b2 = -(dnk * idy * (bn + bk) * 0.5f) + xb2 * (0.25f * idx) * (cn + ck) * 0.5f;
    const float a1m = fminf(a1, 0.f), a1p = fmaxf(a1, 0.f);
    const float a2m = fminf(a2, 0.f), a2p = fmaxf(a2, 0.f);
    const float b1m = fminf(b1, 0.f), b1p = fmaxf(b1, 0.f);
    const float b2m = fminf(b2, 0.f), b2p = fmaxf(b2, 0.f);
    const float d = (a2p - a1m) * idx + (b2p - b1m) * idy;
    float id = 0.f, ww = 0.f, we = 0.f, ws = 0.f, wn = 0.f;
    if (!(fabsf(d) < (float)EPS14)) {
      id = __frcp_rn(d);
      ww = a1p * idx * id;
      we = -(a2m * idx) * id;
      ws = b1p * idy * id;
      wn = -(b2m * idy) * id;
    }
    V.W[k] = ww;
    V.W[N + k] = we;
    V.W[2 * N + k] = ws;
    V.W[3 * N + k] = wn;
    for (int f = 0; f < nf; ++f) V.src[f][k] = (float)(V.delta[f][k] * (double)id);
  }
  __syncthreads();
}

struct AdjOps {
  int k, t;
  bool on;
  float ww, we, ws, wn, src, old;
};

__device__ __forceinline__ void adj_load(AdjOps& o, const SweepGeom& g, int d, int nd, int nx,
                                         size_t N, int pitch, const F32View& V, int f,
                                         bool last_sweep) {
  o.on = false;
  if (d >= nd) return;
  const int v = g.vmin(d) + (int)threadIdx.x;
  if (v > g.vmax(d)) return;
  int i, j;
  g.cell(d, v, i, j);
  const int k = i + nx * j;
  o.on = true;
  o.k = k;
  o.t = i + pitch * j;
  o.ww = V.W[k];
  o.we = V.W[N + k];
  o.ws = V.W[2 * N + k];
  o.wn = V.W[3 * N + k];
  o.src = V.src[f][k];
  if (last_sweep) o.old = V.old[k];
}

// Sweeps one adjoint field held in `ta` (pitched) to convergence.
__device__ inline void f32_adj_sweeps(const PeriodDev& P, const F32View& V, float* ta, int pitch,
                                      int f, SolveShared& sh, int* iters_out, int* status_out) {
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  // Ta = 100 inside, 0 on the boundary (:1368-1380)
  for (size_t k = threadIdx.x; k < N; k += blockDim.x) {
    const int i = (int)(k % nx), j = (int)(k / nx);
    const bool in = i > 0 && i < nx - 1 && j > 0 && j < ny - 1;
    ta[i + (size_t)pitch * j] = in ? 100.f : 0.f;
  }
  __syncthreads();
  int iter, status = ST_NOT_CONVERGED;
  for (iter = 1; iter <= MAXITER_JSE; ++iter) {
    double l1 = 0.0, linf = 0.0, vmax = 0.0;
    for (int s = 0; s < 4; ++s) {
      SweepGeom g;
      g.ilo = 1; g.ihi = nx - 2; g.jlo = 1; g.jhi = ny - 2;
      sweep_dirs(s, g.xdir, g.ydir);
      const int nd = g.ndiag();
      AdjOps cur, nxt;
      adj_load(cur, g, 0, nd, nx, N, pitch, V, f, s == 3);
      for (int d = 0; d < nd; ++d) {
        adj_load(nxt, g, d + 1, nd, nx, N, pitch, V, f, s == 3);
        if (cur.on) {
          const int t = cur.t;
          const float before = ta[t];
          const float nv = cur.src + cur.ww * ta[t - 1] + cur.we * ta[t + 1] +
                           cur.ws * ta[t - pitch] + cur.wn * ta[t + pitch];
          ta[t] = nv;
          if (s == 0) V.old[cur.k] = before;
          if (s == 3) {
            const double dd = fabs((double)nv - (double)cur.old);
            l1 += dd;
            linf = fmax(linf, dd);
            vmax = fmax(vmax, fabs((double)nv));
          }
        }
        __syncthreads();
        cur = nxt;
      }
    }
    double s1 = l1, sm = linf;
    block_sum_max(s1, sm, sh.red);
    double z = 0.0, vm = vmax;
    block_sum_max(z, vm, sh.red);
    s1 = s1 / (double)(nx * ny);
    // reference rule (:1429), or no change beyond the FP32 resolution of the field
    if ((fabs(s1) < TOL_JSE && sm < TOL_JSE) || sm <= vm * 0x1p-21) {
      status = ST_OK;
      break;
    }
  }
  *iters_out = iter > MAXITER_JSE ? MAXITER_JSE : iter;
  *status_out = status;
}

// ---------------------------------------------------------------------------
// The persistent solve kernel
// ---------------------------------------------------------------------------
template <bool SMEM, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) k_batch_fp32(BatchArgs A) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ SolveShared sh;
  __shared__ int next;
  double* colc = reinterpret_cast<double*>(dsm);
  double* cols = colc + A.max_nx;
  float* stau = reinterpret_cast<float*>(cols + A.max_nx);
  double* base = A.ws + (size_t)blockIdx.x * (size_t)A.ws_doubles;
  for (;;) {
    if (threadIdx.x == 0) next = atomicAdd(A.queue, 1);
    __syncthreads();
    const int q = next;
    __syncthreads();
    if (q >= A.nsolve) break;
    const int s = A.order[q];
    const PeriodDev P = A.periods[A.pidx[s]];
    const int nx = P.nx, ny = P.ny;
    const size_t N = (size_t)nx * ny;
    const int pitch = f32_pitch(nx);
    if (threadIdx.x == 0) sh.flag = ST_OK;
    F32View V = carve32(base, N);
    float* tau = SMEM ? stau : V.gtau;
    const double x0 = A.srcx[s] / 180.0 * PI_S, y0 = A.srcy[s] / 180.0 * PI_S;
    f32_setup(P, x0, y0, V, tau, pitch, colc, cols, sh);
    if (sh.status != ST_OK) {
      const int st = sh.status;
      __syncthreads();
      solve_fail(A, P, s, st);
      continue;
    }
    f32_fwd_sweeps(P, V, tau, pitch, sh);
    const int fst = sh.status, fit = sh.iters;
    for (size_t k = threadIdx.x; k < N; k += blockDim.x) {
      const int i = (int)(k % nx), j = (int)(k / nx);
      V.T[k] = (double)tau[i + (size_t)pitch * j] * V.T0d[k];
    }
    if (A.fwd_updates && threadIdx.x == 0) {
      const Box b = sh.box;
      const double frozen = (double)(b.i1 - b.i0 + 1) * (b.j1 - b.j0 + 1);
      A.fwd_updates[s] = (double)fit * 4.0 * ((double)N - frozen);
    }
    __syncthreads();
    tail_receivers(A, P, s, V.T, sh);
    int st = fst;
    if (sh.flag != ST_OK && st == ST_OK) st = sh.flag;
    int aiters = 0;
    if (A.mode >= 2) {
      const int nf = A.mode == 3 ? 2 : 1;
      const int r0 = A.rec_off[s], nr = A.nrec[s];
      for (int f = 0; f < nf; ++f)
        for (size_t k = threadIdx.x; k < N; k += blockDim.x) V.delta[f][k] = 0.0;
      __syncthreads();
      if (threadIdx.x == 0) {
        // sourceAdj = weight*(tekio-tt) (src/measadj.f90:88) and -1.0*weight (:102)
        int e = ST_OK;
        for (int f = 0; f < nf && e == ST_OK; ++f)
          for (int r = 0; r < nr && e == ST_OK; ++r) {
            const double w = A.wgt_eff[r0 + r];
            const double sv = f == 0 ? w * (A.tekio[r0 + r] - A.tt[r0 + r]) : -1.0 * w;
            e = adj_splat(P, V.delta[f], 1, A.recx + r0 + r, A.recy + r0 + r, nullptr, sv);
          }
        if (e != ST_OK) sh.flag = e;
      }
      __syncthreads();
      if (sh.flag != ST_OK && st == ST_OK) st = sh.flag;
      f32_adj_setup(P, V, nf);
      // mask box (:1449-1467), separable, in the caller's degrees
      const double xd0 = A.srcx[s], yd0 = A.srcy[s];
      const double ddx = P.xdeg[1] - P.xdeg[0], ddy = P.ydeg[1] - P.ydeg[0];
      double* ks = A.kcontrib + A.kslot[s];
      double* kd = A.mode == 3 ? A.kcontrib_den + A.kslot[s] : nullptr;
      const double* isv = P.isv + (A.mode == 3 ? N : 0);
      int its[2] = {0, 0};
      for (int f = 0; f < nf; ++f) {
        int ast = ST_OK;
        f32_adj_sweeps(P, V, tau, pitch, f, sh, &its[f], &ast);
        if (ast != ST_OK && st == ST_OK) st = ast;
        double* out = f == 0 ? ks : kd;
        for (size_t k = threadIdx.x; k < N; k += blockDim.x) {
          const int i = (int)(k % nx), j = (int)(k / nx);
          const bool masked = fabs(P.xdeg[i] - xd0) < 1.5 * ddx && fabs(P.ydeg[j] - yd0) < 1.5 * ddy;
          const double v = masked ? 0.0 : (double)tau[i + (size_t)pitch * j];
          out[k] = v * isv[k];
        }
        __syncthreads();
      }
      aiters = its[0] > its[1] ? its[0] : its[1];
      if (A.adj_updates && threadIdx.x == 0)
        A.adj_updates[s] = (double)(its[0] + its[1]) * 4.0 * (nx - 2) * (ny - 2);
    }
    if (threadIdx.x == 0) {
      A.status[s] = st;
      A.fwd_iters[s] = fit;
      A.adj_iters[s] = aiters;
    }
    __syncthreads();
  }
}

// Instantiations: blocks of up to 128 threads (grids whose shorter side is
// <= 128, three resident solves per SM) and up to 512 threads.
template <bool SMEM, int MAXT, int MINB>
static void launch_one(const BatchArgs& a, int grid, int block, cudaStream_t st) {
  cudaFuncSetAttribute(k_batch_fp32<SMEM, MAXT, MINB>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)a.smem_bytes);
  k_batch_fp32<SMEM, MAXT, MINB><<<grid, block, a.smem_bytes, st>>>(a);
}

template <bool SMEM, int MAXT, int MINB>
static int occupancy_one(int block, size_t smem) {
  int n = 0;
  cudaFuncSetAttribute(k_batch_fp32<SMEM, MAXT, MINB>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_fp32<SMEM, MAXT, MINB>, block, smem);
  return n;
}

void launch_batch_fp32(const BatchArgs& a, int grid, int block, cudaStream_t st) {
  if (block <= 128) {
    if (a.smem_tau) launch_one<true, 128, 3>(a, grid, block, st);
    else launch_one<false, 128, 3>(a, grid, block, st);
  } else {
    if (a.smem_tau) launch_one<true, F32_MAX_THREADS, 1>(a, grid, block, st);
    else launch_one<false, F32_MAX_THREADS, 1>(a, grid, block, st);
  }
}

int batch_fp32_max_blocks_per_sm(int block, size_t smem, int smem_tau) {
  if (block <= 128)
    return smem_tau ? occupancy_one<true, 128, 3>(block, smem)
                    : occupancy_one<false, 128, 3>(block, smem);
  return smem_tau ? occupancy_one<true, F32_MAX_THREADS, 1>(block, smem)
                  : occupancy_one<false, F32_MAX_THREADS, 1>(block, smem);
}

}  // namespace sgb
