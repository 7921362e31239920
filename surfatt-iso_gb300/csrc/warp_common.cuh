// warp_common.cuh -- pieces shared by the FP32 warp-per-solve kernels: the
// source locator, the tau = tau_X + delta visit (FP32x2 pairs) and the lane
// exchanges of the row-per-lane wavefront.
#pragma once
#include "kernels.cuh"
#include "solver_fp64.cuh"

namespace sgb {

constexpr unsigned FULL = 0xffffffffu;

struct WSolve {
  int status;
  double fun0;
  Box box;   // frozen source box
  Box mbox;  // mask box (|x-x0| < 1.5 dx, |y-y0| < 1.5 dy)
  int si, sj;  // source cell
};

__device__ __forceinline__ double shfl_d(double v, int src) {
  return __shfl_sync(FULL, v, src);
}


// ---------------------------------------------------------------------------
// setup
// ---------------------------------------------------------------------------
__device__ inline WSolve w_locate(const PeriodDev& P, double x0, double y0, double xd0,
                                  double yd0, int lane) {
  WSolve w;
  const int nx = P.nx, ny = P.ny;
  if (lane == 0) {
    w.status = ST_OK;
    w.fun0 = 0;
    float r1 = 0.f, r2 = 0.f;
    const int i0 = locate_cell(P.xs, nx - 1, P.dx, x0, &r1);
    const int j0 = locate_cell(P.ys, ny - 1, P.dy, y0, &r2);
    if (i0 < 0 || j0 < 0) {
      w.status = ST_BAD_ARG;
      w.si = w.sj = 0;
    } else {
      float w00 = (1 - r1) * (1 - r2), w01 = (1 - r1) * r2, w10 = r1 * (1 - r2), w11 = r1 * r2;
      const size_t k00 = i0 + (size_t)nx * j0;
      w.fun0 = (double)w00 * P.fun[k00] + (double)w01 * P.fun[k00 + nx] +
               (double)w10 * P.fun[k00 + 1] + (double)w11 * P.fun[k00 + nx + 1];
      w.si = i0;
      w.sj = j0;
    }
  }
  w.status = __shfl_sync(FULL, w.status, 0);
  w.fun0 = shfl_d(w.fun0, 0);
  w.si = __shfl_sync(FULL, w.si, 0);
  w.sj = __shfl_sync(FULL, w.sj, 0);
  // frozen box (|x-x0| <= dx, |y-y0| <= dy) and mask box (|x-x0| < 1.5 dx in
  // degrees): the nodes' tests spread over the lanes, then min / max
  int a0 = nx, a1 = -1, b0 = ny, b1 = -1, c0 = nx, c1 = -1, e0 = ny, e1 = -1;
  const double ddx = P.xdeg[1] - P.xdeg[0], ddy = P.ydeg[1] - P.ydeg[0];
  for (int i = lane; i < nx; i += 32) {
    if (fabs((P.xs[i] - x0) / P.dx) <= 1.0) { a0 = min(a0, i); a1 = max(a1, i); }
    if (fabs(P.xdeg[i] - xd0) < 1.5 * ddx) { c0 = min(c0, i); c1 = max(c1, i); }
  }
  for (int j = lane; j < ny; j += 32) {
    if (fabs((P.ys[j] - y0) / P.dy) <= 1.0) { b0 = min(b0, j); b1 = max(b1, j); }
    if (fabs(P.ydeg[j] - yd0) < 1.5 * ddy) { e0 = min(e0, j); e1 = max(e1, j); }
  }
  w.box = Box{__reduce_min_sync(FULL, a0), __reduce_max_sync(FULL, a1),
              __reduce_min_sync(FULL, b0), __reduce_max_sync(FULL, b1)};
  w.mbox = Box{__reduce_min_sync(FULL, c0), __reduce_max_sync(FULL, c1),
               __reduce_min_sync(FULL, e0), __reduce_max_sync(FULL, e1)};
  const Box& b = w.box;
  if (w.status == ST_OK && b.i0 <= b.i1 && b.j0 <= b.j1 &&
      (b.i0 == 0 || b.i1 == nx - 1 || b.j0 == 0 || b.j1 == ny - 1))
    w.status = ST_SOURCE_ON_BOUNDARY;
  return w;
}

// ---------------------------------------------------------------------------
// forward sweep visit (tau = tau_X + delta form, FP32x2 pairs)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 wbc(float x) { return make_float2(x, x); }
__device__ __forceinline__ float2 wadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 wmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 wfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 wneg(float2 a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ float w_pick(float r, float chx, float chy, float sx, float sy, bool ok) {
  const bool cx = sx > 0.f ? chx >= 0.f : chx <= 0.f;
  const bool cy = sy > 0.f ? chy >= 0.f : chy <= 0.f;
  return (ok && cx && cy) ? r : __int_as_float(0x7f800000);
}

__device__ __forceinline__ float w_two_sided(float2 px, float2 tX, float2 U0, float py, float tY,
                                             float sY, float gy, float cy, float a, float b,
                                             float c, float f2, bool okx, bool oky) {
  const float2 A = wfma(px, wfma(wbc(a), px, wbc(-2.f * c * py)), wbc(b * py * py));
  const float2 bx = wfma(wbc(a), px, wbc(-c * py));
  const float2 by = wfma(wbc(-c), px, wbc(b * py));
  const float2 V0 = wfma(wbc(gy), tX, wmul(wbc(-sY * cy), wadd(tX, wbc(-tY))));
  const float2 CU = wfma(wbc(a), U0, wmul(wbc(-c), V0));
  const float2 CV = wfma(wbc(b), V0, wmul(wbc(-c), U0));
  const float2 C = wfma(U0, CU, wfma(V0, CV, wbc(-f2)));
  const float2 H = wfma(bx, U0, wmul(by, V0));
  const float2 D = wfma(H, H, wmul(wneg(A), C));
  const bool vx = okx && D.x >= 0.f, vy = oky && D.y >= 0.f;
  const float2 sq = make_float2(fsqrt_fast(D.x), fsqrt_fast(D.y));
  const float2 ia = make_float2(frcp_fast(A.x), frcp_fast(A.y));
  const float2 d1 = wmul(wadd(sq, wneg(H)), ia);
  const float2 d2 = wmul(wadd(wneg(sq), wneg(H)), ia);
  const float2 x1 = wfma(bx, d1, CU), y1 = wfma(by, d1, CV);
  const float2 x2 = wfma(bx, d2, CU), y2 = wfma(by, d2, CV);
  const float2 r1 = wadd(tX, d1), r2 = wadd(tX, d2);
  const float sy = -sY;
  float m = w_pick(r1.x, x1.x, y1.x, 1.f, sy, vx);
  m = fminf(m, w_pick(r2.x, x2.x, y2.x, 1.f, sy, vx));
  m = fminf(m, w_pick(r1.y, x1.y, y1.y, -1.f, sy, vy));
  m = fminf(m, w_pick(r2.y, x2.y, y2.y, -1.f, sy, vy));
  return m;
}

__device__ __forceinline__ float w_one_sided(float2 p, float2 tnb, float2 t0nb, float g,
                                             float dis, float t0, bool okx, bool oky) {
  const float2 ip = make_float2(frcp_fast(p.x), frcp_fast(p.y));
  const float2 gt = wmul(wbc(g), tnb);
  const float2 r1 = wfma(wadd(wbc(dis), wneg(gt)), ip, tnb);
  const float2 r2 = wfma(wadd(wbc(-dis), wneg(gt)), ip, tnb);
  const float2 lim = wmul(tnb, t0nb), half = wmul(tnb, wbc(0.5f));
  const float2 s1 = wmul(r1, wbc(t0)), s2 = wmul(r2, wbc(t0));
  const float inf = __int_as_float(0x7f800000);
  float m = (okx && s1.x >= lim.x && r1.x > half.x) ? r1.x : inf;
  m = fminf(m, (okx && s2.x >= lim.x && r2.x > half.x) ? r2.x : inf);
  m = fminf(m, (oky && s1.y >= lim.y && r1.y > half.y) ? r1.y : inf);
  m = fminf(m, (oky && s2.y >= lim.y && r2.y > half.y) ? r2.y : inf);
  return m;
}

// Operands of one forward visit, loaded a step ahead.  The downstream
// neighbours are not loaded here: the logical east cell (u+1, v) is this
// band's next cell and the logical north cell (u, v+1) is the next cell of
// the lane above, so their old tau and T0 come from `nxt` (own register or
// __shfl_down); the south T0 comes from the lane below (__shfl_up).
struct WFwd {
  bool on, frz;
  float own, old;  // old tau of the cell; tau at the start of the iteration
  float t0, gx, gy;
  float4 pa;       // a, b, c, fun^2
  float dsx, dsy;
};

// Per band: the next-step value / T0 of row v+1 (lane above; lane 0 of band
// m+1 for lane 31), one shuffle each.
template <int MB>
__device__ __forceinline__ float w_above_own(const WFwd (&x)[MB], int m, int lane) {
  const float offer = lane == 0 ? x[m + 1 < MB ? m + 1 : m].own : x[m].own;
  return __shfl_sync(FULL, offer, (lane + 1) & 31);
}
// The same for a per-band value array.
template <int MB>
__device__ __forceinline__ float w_above(const float (&x)[MB], int m, int lane) {
  const float offer = lane == 0 ? x[m + 1 < MB ? m + 1 : m] : x[m];
  return __shfl_sync(FULL, offer, (lane + 1) & 31);
}
template <int MB>
__device__ __forceinline__ float w_above_t0(const WFwd (&x)[MB], int m, int lane) {
  const float offer = lane == 0 ? x[m + 1 < MB ? m + 1 : m].t0 : x[m].t0;
  return __shfl_sync(FULL, offer, (lane + 1) & 31);
}


// Visit with logical neighbours mapped to the physical W/E/S/N of the
// reference's update.  west/south: new values; east/north: old values.
__device__ __forceinline__ float wf_visit(const WFwd& o, float west, float east, float south,
                                          float north, float t0w, float t0e, float t0s, float t0n,
                                          bool hasw, bool hass, bool hase, bool hasn, int xdir,
                                          int ydir, float idx, float idy) {
  const float tw = xdir > 0 ? west : east, te = xdir > 0 ? east : west;
  const float ts = ydir > 0 ? south : north, tn = ydir > 0 ? north : south;
  const bool hw = xdir > 0 ? hasw : hase, he = xdir > 0 ? hase : hasw;
  const bool hs = ydir > 0 ? hass : hasn, hn = ydir > 0 ? hasn : hass;
  const float t0wp = xdir > 0 ? t0w : t0e, t0ep = xdir > 0 ? t0e : t0w;
  const float t0sp = ydir > 0 ? t0s : t0n, t0np = ydir > 0 ? t0n : t0s;
  const float t0 = o.t0, gx = o.gx, gy = o.gy;
  const float a = o.pa.x, b = o.pa.y, c = o.pa.z, f2 = o.pa.w;
  // T0/dx, T0/dy rounded once; the sums below are explicit roundings so that
  // no compiler contraction changes a result between kernel builds
  const float cx = __fmul_rn(t0, idx), cy = __fmul_rn(t0, idy);
  const float pyp = __fadd_rn(gy, cy), pym = __fsub_rn(gy, cy);
  const float2 px = make_float2(__fadd_rn(gx, cx), __fsub_rn(gx, cx));
  const float2 tX = make_float2(tw, te);
  const float2 U0 = wmul(wbc(gx), tX);
  float m = w_two_sided(px, tX, U0, pyp, ts, -1.f, gy, cy, a, b, c, f2, hw && hs, he && hs);
  m = fminf(m, w_two_sided(px, tX, U0, pym, tn, 1.f, gy, cy, a, b, c, f2, hw && hn, he && hn));
  m = fminf(m, w_one_sided(px, tX, make_float2(t0wp, t0ep), gx, o.dsx, t0, hw, he));
  m = fminf(m, w_one_sided(make_float2(pyp, pym), make_float2(ts, tn),
                           make_float2(t0sp, t0np), gy, o.dsy, t0, hs, hn));
  return fminf(o.own, m);
}

// Per band: the previous-step value of row v-1 (lane below; lane 31 of band
// m-1 for lane 0), one shuffle: lane 31 offers band m-1's value, the others
// band m's.
template <int MB>
__device__ __forceinline__ float w_below(const float (&x)[MB], int m, int lane) {
  const float offer = lane == 31 ? x[m > 0 ? m - 1 : 0] : x[m];
  return __shfl_sync(FULL, offer, (lane + 31) & 31);
}

// Value of row v-1 held by the lane below (lane 31 of the band below for lane 0).
template <int MB>
__device__ __forceinline__ void w_from_below(const float (&x)[MB], float (&out)[MB], int lane) {
#pragma unroll
  for (int m = 0; m < MB; ++m) {
    const float up = __shfl_up_sync(FULL, x[m], 1);
    const float wr = __shfl_sync(FULL, x[m > 0 ? m - 1 : 0], 31);
    out[m] = lane > 0 ? up : wr;
  }
}

// Value of row v+1 held by the lane above (lane 0 of the band above for lane 31).
template <int MB>
__device__ __forceinline__ void w_from_above(const float (&x)[MB], float (&out)[MB], int lane) {
#pragma unroll
  for (int m = 0; m < MB; ++m) {
    const float dn = __shfl_down_sync(FULL, x[m], 1);
    const float wr = __shfl_sync(FULL, x[m + 1 < MB ? m + 1 : m], 0);
    out[m] = lane < 31 ? dn : wr;
  }
}

// ---------------------------------------------------------------------------
// T0 = R fun0 d and its gradient.  d = 2 asin(sqrt(h)), h = sin^2(dy/2) +
// cos y cos y0 sin^2(dx/2), is the reference's acos(sin y sin y0 + cos y
// cos y0 cos dx) (src/eikon_solver_2d.f90:847-856) without its cancellation;
// sin d = 2 sqrt(h (1-h)).  Within two cells of the source the reference's
// own FP64 expressions are used.
// ---------------------------------------------------------------------------
struct T0Src {
  double x0, y0, cy0d, sy0d, fun0;
  float rff, cy0;
  int si, sj;
};

struct T0Row {
  float shy, chy, cy, sy;
};

__device__ inline T0Src t0_source(const WSolve& w, double x0, double y0) {
  T0Src s;
  s.x0 = x0;
  s.y0 = y0;
  s.cy0d = cos(y0);
  s.sy0d = sin(y0);
  s.fun0 = w.fun0;
  s.rff = (float)(R_EARTH * w.fun0);
  s.cy0 = (float)s.cy0d;
  s.si = w.si;
  s.sj = w.sj;
  return s;
}

__device__ inline T0Row t0_row(const PeriodDev& P, const T0Src& s, int j) {
  T0Row r;
  const float hy = (float)((P.ys[j] - s.y0) * 0.5);
  r.shy = sinf(hy);
  r.chy = cosf(hy);
  r.cy = (float)P.cosy[j];
  r.sy = (float)P.siny[j];
  return r;
}

// {T0, T0x, T0y, 0} of node (i, j); shx, chx: sin and cos of half the
// longitude offset of column i.
__device__ inline float4 t0_cell(const PeriodDev& P, const T0Src& s, const T0Row& r, int i, int j,
                                 float shx, float chx) {
  float t0, gx, gy;
  if (abs(i - s.si) <= 2 && abs(j - s.sj) <= 2) {
    const double cyy = P.cosy[j], syy = P.siny[j];
    const double cdx = cos(P.xs[i] - s.x0), sdx = sin(P.xs[i] - s.x0);
    const double tmp = syy * s.sy0d + cyy * s.cy0d * cdx;
    double cl = tmp < 1.0 ? tmp : 1.0;
    cl = cl > -1.0 ? cl : -1.0;
    const double td = acos(cl) * R_EARTH * s.fun0;
    double tx = 0, ty = 0;
    if (td != 0) {
      const double rs = 1.0 / sqrt(1 - tmp * tmp);
      tx = -(rs * cyy * s.cy0d * (-1.0) * sdx * R_EARTH * s.fun0);
      ty = -(rs * (cyy * s.sy0d - syy * s.cy0d * cdx) * R_EARTH * s.fun0);
    }
    t0 = (float)td;
    gx = (float)tx;
    gy = (float)ty;
  } else {
    const float h = __fadd_rn(__fmul_rn(r.shy, r.shy), __fmul_rn(r.cy * s.cy0, shx * shx));
    const float sh = sqrtf(h);
    const float d = 2.f * asinf(fminf(sh, 1.f));
    const float sind = 2.f * sh * sqrtf(fmaxf(1.f - h, 0.f));
    t0 = s.rff * d;
    if (sind > 0.f) {
      const float inv = s.rff / sind;
      gx = inv * r.cy * s.cy0 * (2.f * shx * chx);
      // -(cos y sin y0 - sin y cos y0 cos dx) = -(sin(y0-y) + 2 sin y cos y0 sin^2(dx/2))
      gy = -inv * __fadd_rn(__fmul_rn(-2.f * r.shy, r.chy),
                            __fmul_rn(2.f * r.sy * s.cy0, shx * shx));
    } else {
      gx = 0.f;
      gy = 0.f;
    }
  }
  return make_float4(t0, gx, gy, 0.f);
}

// ---------------------------------------------------------------------------
// adjoint arithmetic shared by the warp kernels, written with explicit
// roundings (no compiler contraction)
// ---------------------------------------------------------------------------
// Ta = src + ww*Ta_W + we*Ta_E + ws*Ta_S + wn*Ta_N
__device__ __forceinline__ float adj_update(float src, float4 W, float tw, float te, float ts,
                                            float tn) {
  return __fmaf_rn(W.w, tn, __fmaf_rn(W.z, ts, __fmaf_rn(W.y, te, __fmaf_rn(W.x, tw, src))));
}

// Weights {ww, we, ws, wn} and 1/d of an interior node from T at its 3x3
// stencil (Tc: centre; w/e/s/n; wn, ws, en, es corners) and the metric
// records {a, b, c, -} of the node and its four neighbours
// (src/eikon_solver_2d.f90:1348-1370).
__device__ inline float adj_weights(float Tk, float Tw, float Te, float Ts, float Tn, float Twn,
                                    float Tws, float Ten, float Tes, float4 pk, float4 pw,
                                    float4 pe, float4 ps, float4 pn, float idx, float idy,
                                    float4* W) {
  const float hx = 0.25f * idy, hy = 0.25f * idx;
  // a1 = -((Tk-Tw) idx (a_k+a_w)/2) + (Tn - Ts + Twn - Tws) idy/4 (c_k+c_w)/2, etc.
  const float a1 = __fadd_rn(-(__fmul_rn(__fmul_rn(__fmul_rn(Tk - Tw, idx), pk.x + pw.x), 0.5f)),
                             __fmul_rn(__fmul_rn(__fmul_rn(Tn - Ts + Twn - Tws, hx), pk.z + pw.z), 0.5f));
  const float a2 = __fadd_rn(-(__fmul_rn(__fmul_rn(__fmul_rn(Te - Tk, idx), pe.x + pk.x), 0.5f)),
                             __fmul_rn(__fmul_rn(__fmul_rn(Ten - Tes + Tn - Ts, hx), pe.z + pk.z), 0.5f));
  const float b1 = __fadd_rn(-(__fmul_rn(__fmul_rn(__fmul_rn(Tk - Ts, idy), pk.y + ps.y), 0.5f)),
                             __fmul_rn(__fmul_rn(__fmul_rn(Te - Tw + Tes - Tws, hy), pk.z + ps.z), 0.5f));
  const float b2 = __fadd_rn(-(__fmul_rn(__fmul_rn(__fmul_rn(Tn - Tk, idy), pn.y + pk.y), 0.5f)),
                             __fmul_rn(__fmul_rn(__fmul_rn(Ten - Twn + Te - Tw, hy), pn.z + pk.z), 0.5f));
  const float a1m = fminf(a1, 0.f), a1p = fmaxf(a1, 0.f);
  const float a2m = fminf(a2, 0.f), a2p = fmaxf(a2, 0.f);
  const float b1m = fminf(b1, 0.f), b1p = fmaxf(b1, 0.f);
  const float b2m = fminf(b2, 0.f), b2p = fmaxf(b2, 0.f);
  const float d = __fadd_rn(__fmul_rn(a2p - a1m, idx), __fmul_rn(b2p - b1m, idy));
  float id = 0.f;
  *W = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!(fabsf(d) < (float)EPS14)) {
    id = __frcp_rn(d);
    *W = make_float4(__fmul_rn(a1p * idx, id), __fmul_rn(-(a2m * idx), id),
                     __fmul_rn(b1p * idy, id), __fmul_rn(-(b2m * idy), id));
  }
  return id;
}

// Adjoint sources of one solve: weight*(tekio-tt) for field 0
// (src/measadj.f90:88) and -weight for field 1 (:102), each splat
// bilinearly over the receiver's cell divided by the cell area
// (src/eikon_solver_2d.f90:1328-1336) and scaled by the cell's 1/d.  Called
// by all 32 lanes of one warp.  The lanes evaluate 32 receivers at a time
// (cell search, cos, the FP64 quotients: the costly part, which a single
// lane would run at 1/32 of the FP64 pipe); lane 0 then adds the
// contributions in receiver order, so every cell's sum is the sequential
// one.  A receiver outside the grid stops field 0 there, skips field 1 and
// returns ST_BAD_ARG, as the sequential loop over fields and receivers
// does.  `ix(i, j)` maps a node to its index in `sf0`, `sf1` and `id`.
template <class Ix>
__device__ inline int adj_sources_warp(const BatchArgs& A, const PeriodDev& P, int r0, int nr,
                                       int nf, float* sf0, float* sf1, const float* id, Ix ix,
                                       int lane, int st) {
  if (st == ST_BAD_ARG) return st;
  const int nx = P.nx, ny = P.ny;
  auto cell = [&](int r, int* i0, int* j0, float* r1, float* r2, double* yr) {
    const double xr = A.recx[r0 + r] / 180.0 * PI_S;
    *yr = A.recy[r0 + r] / 180.0 * PI_S;
    *i0 = locate_cell(P.xs, nx, P.dx, xr, r1);
    *j0 = locate_cell(P.ys, ny, P.dy, *yr, r2);
  };
  // the first receiver outside the grid (nr: none)
  int n0 = nr;
  for (int rb = 0; rb < nr; rb += 32) {
    bool out = false;
    if (rb + lane < nr) {
      int i0, j0;
      float r1, r2;
      double yr;
      cell(rb + lane, &i0, &j0, &r1, &r2, &yr);
      out = i0 < 0 || j0 < 0;
    }
    const unsigned m = __ballot_sync(FULL, out);
    if (m) {
      n0 = rb + __ffs(m) - 1;
      break;
    }
  }
  const bool two = nf == 2 && n0 == nr;
  for (int rb = 0; rb < n0; rb += 32) {
    int i0 = 0, j0 = 0;
    float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
    if (rb + lane < n0) {
      const int r = rb + lane;
      float r1 = 0.f, r2 = 0.f;
      double yr;
      cell(r, &i0, &j0, &r1, &r2, &yr);
      const double wt = A.wgt_eff[r0 + r];
      const double sv0 = wt * (A.tekio[r0 + r] - A.tt[r0 + r]), sv1 = -1.0 * wt;
      const double den = P.dx * R_EARTH * cos(yr) * P.dy * R_EARTH;
      // corner c = (i0 + c/2, j0 + c%2): sv * wx * wy / den, left to right
      const double wx[2] = {(double)(1 - r1), (double)r1}, wy[2] = {(double)(1 - r2), (double)r2};
      const bool has[4] = {true, j0 + 1 < ny, i0 + 1 < nx, i0 + 1 < nx && j0 + 1 < ny};
#pragma unroll
      for (int c = 0; c < 4; ++c)
        if (has[c]) {
          const float d = id[ix(i0 + (c >> 1), j0 + (c & 1))];
          c0[c] = __fmul_rn((float)(sv0 * wx[c >> 1] * wy[c & 1] / den), d);
          if (two) c1[c] = __fmul_rn((float)(sv1 * wx[c >> 1] * wy[c & 1] / den), d);
        }
    }
    const int cnt = min(32, n0 - rb);
    for (int l = 0; l < cnt; ++l) {
      const int i = __shfl_sync(FULL, i0, l), j = __shfl_sync(FULL, j0, l);
      float a0[4], a1[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        a0[c] = __shfl_sync(FULL, c0[c], l);
        a1[c] = two ? __shfl_sync(FULL, c1[c], l) : 0.f;
      }
      if (lane == 0) {
        const bool has[4] = {true, j + 1 < ny, i + 1 < nx, i + 1 < nx && j + 1 < ny};
#pragma unroll
        for (int c = 0; c < 4; ++c)
          if (has[c]) {
            const int k = ix(i + (c >> 1), j + (c & 1));
            sf0[k] = __fadd_rn(sf0[k], a0[c]);
            if (two) sf1[k] = __fadd_rn(sf1[k], a1[c]);
          }
      }
    }
  }
  return n0 < nr ? ST_BAD_ARG : st;
}

}  // namespace sgb
