// kernels_fp32w.cu -- FP32-factored batched solve, one warp per (period,
// source) solve for grids of at most 128 rows; for grids of up to 512 rows
// either a team of up to four warps (one block, 128 rows each) or one warp
// sweeping the same 128-row strips one after another (same results, bit for
// bit: fewer warp-steps per solve, twice the steps in a row).
//
// Wavefront without block barriers.  In each of the four sweeps, lane l owns
// the logical rows v = l + 32*m (m < MB) and at step t visits the cell
// u = t - v of each of its rows.  Of the four stencil neighbours of (u, v),
// the two already updated in this sweep come from registers: (u-1, v) is the
// lane's own previous result, (u, v-1) the previous result of the lane below
// (one __shfl_up; lane 0 takes lane 31's value of the band below).  The two
// not yet updated, (u+1, v) and (u, v+1), are read from global memory a step
// ahead (they are rewritten only after that read), together with the cell's
// operands.  Visiting u = t - v for every row reproduces the reference's
// in-place Gauss-Seidel order exactly (a cell's up-/left-stream neighbours
// are final, its down-/right-stream ones are old), with one __syncwarp() per
// step instead of a block barrier and no shared memory, so a GPU holds one
// resident solve per warp (register-bound) rather than per block.
//
// Precision (the FP32-factored form): tau and the adjoint fields are FP32;
// the sweep update is the tau = tau_X + delta form of the block kernel.  T0
// and its gradient come from the haversine form of the reference's
// great-circle distance (well conditioned at small distances) in FP32, and
// in FP64 with the reference's own formula within two cells of the source.
// Misfit, receiver times, the convergence decisions (FP64 reduction of the
// lanes' partial sums) and the per-period kernel sums are FP64.
#include "warp_common.cuh"

namespace sgb {

// A solve's team: the NW warps of one block (NW = 1: the warp alone, one
// warp per block).  tid runs over the team, wid is the warp's rank in it.
template <int NW>
struct Tm {
  int tid, lane, wid;
};

template <int NW>
__device__ __forceinline__ Tm<NW> this_team() {
  Tm<NW> t;
  t.lane = (int)(threadIdx.x & 31);
  t.tid = NW == 1 ? t.lane : (int)threadIdx.x;
  t.wid = NW == 1 ? 0 : (int)(threadIdx.x >> 5);
  return t;
}

template <int NW>
__device__ __forceinline__ void tsync() {
  if (NW == 1) __syncwarp();
  else __syncthreads();
}

// Every thread of the team receives thread 0's value.
template <int NW>
__device__ __forceinline__ int tbcast(int v) {
  if (NW == 1) return __shfl_sync(FULL, v, 0);
  __shared__ int b;
  __syncthreads();
  if (threadIdx.x == 0) b = v;
  __syncthreads();
  return b;
}

// Sum (a) and maxima (b, c) over the team: within each warp by the xor
// tree, then over the warps in order (deterministic).
template <int NW>
__device__ __forceinline__ void tsum_max2(double& a, double& b, double& c) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(FULL, a, o);
    b = fmax(b, __shfl_xor_sync(FULL, b, o));
    c = fmax(c, __shfl_xor_sync(FULL, c, o));
  }
  if (NW == 1) return;
  __shared__ double r[3][NW > 1 ? NW : 1];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) {
    r[0][wid] = a;
    r[1][wid] = b;
    r[2][wid] = c;
  }
  __syncthreads();
  a = 0.0;
  b = 0.0;
  c = 0.0;
  for (int w = 0; w < NW; ++w) {
    a += r[0][w];
    b = fmax(b, r[1][w]);
    c = fmax(c, r[2][w]);
  }
}


// Strips of one warp (at most a team's warps): each strip's partial sums
// reduced as a team reduces a warp's (over the lanes by the xor tree, in
// FP64) and added to the iteration's total in strip order, as the team adds
// its warps' -- the same bits as a team's reduction.
constexpr int kMaxStrips = 4;

__device__ __forceinline__ void w_strip_add(double& acc, float v) {
  double x = (double)v;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
  acc += x;
}

__device__ __forceinline__ double w_warp_max(double b) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) b = fmax(b, __shfl_xor_sync(FULL, b, o));
  return b;
}

// Workspace per warp slot: W (float4 adjoint weights), 4N floats of
// forward state from R, old, 1/d, two scaled adjoint sources (4 bytes each
// per cell), per-column half-angle sines and cosines.  The forward state is
// laid out one of two ways:
//   separate (one-warp kernel):  G = {T0x, T0y} (float2), T0, tau;
//   paired (strips and teams):   TT = {T0, tau} (float2), G.
// A row's forward sweep reads four operand streams with the separate
// layout and three with the paired one; a tall grid's latency-bound strips
// gain from the fewer L1 lines (config 4: 159 -> 154 ms), the one-warp
// kernel does not (17.2 -> 17.4 ms on config 2), so each kernel keeps the
// layout it is faster with (all results are the same bits).
long long batch_fp32w_ws_doubles(long long N) {
  const long long floats = 4 * N + 4 * N + 4 * N + 2 * 4096;  // W, R, old / 1/d / sources, col
  long long d = (floats + 1) / 2 + 64;
  return (d + 31) / 32 * 32;  // keep every slot 256-byte aligned
}

struct WSlot {
  float4* W;
  float* R;    // start of the forward state (4N floats)
  float2* TT;  // paired: {T0, tau} per cell (null when separate)
  float2* G;   // {T0x, T0y} per cell
  float* T0;   // separate: T0, tau per cell (null when paired)
  float* tau;
  float* old;
  float* id;
  float* src[2];
  float* col;  // per column sin and cos of half the longitude offset (2 * nx)
};

__device__ inline WSlot wcarve(double* base, size_t N, bool pair) {
  WSlot V;
  V.W = reinterpret_cast<float4*>(base);
  V.R = reinterpret_cast<float*>(V.W + N);
  if (pair) {
    V.TT = reinterpret_cast<float2*>(V.R);
    V.G = V.TT + N;
    V.T0 = V.tau = nullptr;
  } else {
    V.TT = nullptr;
    V.G = reinterpret_cast<float2*>(V.R);
    V.T0 = reinterpret_cast<float*>(V.G + N);
    V.tau = V.T0 + N;
  }
  V.old = V.R + 4 * N;
  V.id = V.old + N;
  V.src[0] = V.id + N;
  V.src[1] = V.src[0] + N;
  V.col = V.src[1] + N;
  return V;
}

// {T0, tau} of cell k in the kernel's layout
template <bool PAIR>
__device__ __forceinline__ float2 w_t0tau(const WSlot& V, size_t k) {
  if constexpr (PAIR) return V.TT[k];
  return make_float2(V.T0[k], V.tau[k]);
}


// T0 and (T0x, T0y) of every cell; tau initialised (1 in the frozen box).
template <int NW, bool PAIR>
__device__ inline void w_t0(const PeriodDev& P, double x0, double y0, const WSolve& w,
                            const WSlot& V, const Tm<NW>& T) {
  const int nx = P.nx, ny = P.ny, lane = T.lane;
  const T0Src src = t0_source(w, x0, y0);
  for (int i = T.tid; i < nx; i += 32 * NW) {
    const float hx = (float)((P.xs[i] - x0) * 0.5);
    V.col[i] = sinf(hx);
    V.col[nx + i] = cosf(hx);
  }
  tsync<NW>();
  for (int j = T.wid; j < ny; j += NW) {  // rows by warp, columns by lane
    const T0Row row = t0_row(P, src, j);
    for (int i = lane; i < nx; i += 32) {
      const size_t k = i + (size_t)nx * j;
      const float4 c = t0_cell(P, src, row, i, j, V.col[i], V.col[nx + i]);
      const float tau0 = w.box.has(i, j) ? 1.0f : 10.0f;
      if constexpr (PAIR) {
        V.TT[k] = make_float2(c.x, tau0);
      } else {
        V.T0[k] = c.x;
        V.tau[k] = tau0;
      }
      V.G[k] = make_float2(c.y, c.z);
    }
  }
  tsync<NW>();
}


// The sweep's constants of one lane row (logical row v of the sweep's
// frame, physical row j): the cell visited at step t is on the grid when
// 0 <= t - lo < nx and is then cell kb + xdir * t; it is frozen when
// 0 <= t - flo <= flen (flo far away for a row outside the frozen box).
struct WRow {
  int lo, kb, flo;
  bool hass, hasn;  // the row has a south / north neighbour
};

__device__ __forceinline__ WRow w_row(int v, int nx, int ny, int xdir, int ydir, const Box& box) {
  WRow r;
  constexpr int kFar = 1 << 29;
  if (v >= ny) {
    r.lo = kFar;
    r.kb = 0;
    r.flo = kFar;
    r.hass = r.hasn = false;
    return r;
  }
  const int j = ydir > 0 ? v : ny - 1 - v;
  r.lo = v;
  r.kb = nx * j + (xdir > 0 ? -v : nx - 1 + v);
  const bool rib = box.i0 <= box.i1 && box.j0 <= j && j <= box.j1;
  r.flo = rib ? v + (xdir > 0 ? box.i0 : nx - 1 - box.i1) : kFar;
  r.hass = v > 0;
  r.hasn = v < ny - 1;
  return r;
}

// Iterations it0 .. it1 (1-based; the reference runs 1 .. MaxIter): status
// ST_OK and the iteration count when one of them converges, otherwise
// ST_NOT_CONVERGED and it1.
//
// Per band, a lane holds three kinds of operands.  The values it exchanges
// with its neighbours -- old tau and T0 of its cell at steps t and t + 1 --
// sit in a ring loaded two steps ahead (a cell is written only at its own
// visit, so an early read sees the value a read at the visit would).  The
// cell constants of step t (T0 gradient, metric and slowness record,
// one-sided terms, iteration-start tau) are loaded into the band's
// registers right after the band's visit of step t - 1 (PF = 1: they have a
// whole step to arrive and are never copied) or at the visit itself
// (PF = 0: fewer live registers).  Row constants (WRow) are computed once
// per sweep, so a step costs a few integer operations per band.
template <int MB, int PF, int NW, bool ST>
__device__ inline void w_fwd_sweeps(const PeriodDev& P, const WSlot& V, const WSolve& w,
                                    const Tm<NW>& T, int it0, int it1, int* status_out,
                                    int* iters_out) {
  static_assert(!ST || NW == 1, "strips are swept by one warp");
  const int nx = P.nx, ny = P.ny, lane = T.lane;
  const float idx = (float)(1.0 / P.dx), idy = (float)(1.0 / P.dy);
  const int nsteps = nx + ny - 1;
  constexpr bool PAIR = ST || NW > 1;  // this kernel's workspace layout (wcarve)
  const float2* const TT = V.TT;  // paired: {T0, tau}
  const float* const T0a = V.T0;  // separate
  const float* const tau = V.tau;
  const float2* const G = V.G;    // {T0x, T0y}
  // old tau (own) and T0 of cell k
  auto ld_pt = [&](int k, float& own, float& t0) {
    if constexpr (PAIR) {
      const float2 q = TT[k];
      own = q.y;
      t0 = q.x;
    } else {
      own = tau[k];
      t0 = T0a[k];
    }
  };
  const float4* const PA = P.p4a;
  const float2* const PB = reinterpret_cast<const float2*>(P.p4b);  // {disx, disy} at 4k
  const int flen = w.box.i1 > w.box.i0 ? w.box.i1 - w.box.i0 : 0;
  // Teams: warp w owns the rows vb .. vb + 32 MB - 1.  The south neighbour
  // of its first row is the last row of warp w-1, visited a step earlier:
  // it comes through a shared slot (double-buffered by step parity, one
  // team barrier per step).  The north neighbour of its last row is the
  // first row of warp w+1, visited a step later: its old value is read from
  // memory a step ahead (that cell is rewritten two steps later).
  //
  // Strips (ST): one warp sweeps the team's row blocks one after another,
  // strip p being the rows a team's warp p owns.  When strip p is swept,
  // strip p-1 is final for this sweep and strip p+1 not yet touched, so the
  // south neighbours of its first row (new values) and the north
  // neighbours of its last row (old values) are both in memory, a step
  // ahead; every visit sees the neighbour values it sees in a team, and
  // the per-strip partial sums are reduced in the team's order, so the
  // results are a team's, bit for bit, without the team's barrier per step.
  const int nstrip = ST ? (ny + 32 * MB - 1) / (32 * MB) : 1;
  __shared__ float xs_val[2][NW > 1 ? NW : 1], xs_t0[2][NW > 1 ? NW : 1];
  int iter, status = ST_NOT_CONVERGED;
  for (iter = it0; iter <= it1; ++iter) {
    float l1 = 0.f, lmax = 0.f;
    double l1acc = 0.0;  // strips, last sweep: the strips' reduced sums so far
    for (int s = 0; s < 4; ++s) {
      int xdir, ydir;
      sweep_dirs(s, xdir, ydir);
      const bool last = s == 3;
     for (int sp = 0; sp < nstrip; ++sp) {
      const int vb = 32 * MB * (ST ? sp : T.wid);
      const int vtop = vb + 32 * MB - 1;
      const bool top = (NW > 1 || ST) && lane == 31 && (ST ? vtop + 1 < ny : T.wid < NW - 1);
      const bool bot = (NW > 1 || ST) && lane == 0 && (ST ? sp > 0 : T.wid > 0);
      // a strip's own steps; a team's warps step together over the grid's
      const int tbeg = ST ? vb : 0;
      const int tend = ST ? min(vtop, ny - 1) + nx : nsteps;
      if (ST) l1 = 0.f;
      WRow R[MB];
#pragma unroll
      for (int m = 0; m < MB; ++m) R[m] = w_row(vb + lane + 32 * m, nx, ny, xdir, ydir, w.box);
      // old tau and T0 of band m's cell at step tt (0 off the grid)
      auto exch = [&](int m, int tt, float& own, float& t0) {
        own = 0.f;
        t0 = 0.f;
        if ((unsigned)(tt - R[m].lo) < (unsigned)nx) {
          ld_pt(R[m].kb + xdir * tt, own, t0);
        }
      };
      // the cell constants of band m at step tt
      float gx[MB], gy[MB], dsx[MB], dsy[MB], old[MB];
      float4 pa[MB];
      auto heavy = [&](int m, int tt) {
        if ((unsigned)(tt - R[m].lo) < (unsigned)nx) {
          const int k = R[m].kb + xdir * tt;
          const float2 g = G[k];
          gx[m] = g.x;
          gy[m] = g.y;
          pa[m] = PA[2 * k];
          const float2 d = PB[4 * k];
          dsx[m] = d.x;
          dsy[m] = d.y;
          if (last) old[m] = V.old[k];
        }
      };
      // old tau and T0 of the cell north of the top row at step tt
      auto north_of_top = [&](int tt, float& own, float& t0) {
        const int u = tt - vtop;
        own = 0.f;
        t0 = 0.f;
        if (u >= 0 && u < nx && vtop + 1 < ny) {
          const int k = (xdir > 0 ? u : nx - 1 - u) + nx * (ydir > 0 ? vtop + 1 : ny - 2 - vtop);
          ld_pt(k, own, t0);
        }
      };
      // strips: new tau and T0 of the cell south of the bottom row at step
      // tt (the strip below visited it at step tt - 1)
      auto south_of_bot = [&](int tt, float& own, float& t0) {
        const int u = tt - vb;
        own = 0.f;
        t0 = 0.f;
        if (u >= 0 && u < nx && vb >= 1) {
          const int k = (xdir > 0 ? u : nx - 1 - u) + nx * (ydir > 0 ? vb - 1 : ny - vb);
          ld_pt(k, own, t0);
        }
      };
      // exchange ring: steps t (x0), t + 1 (x1), t + 2 (x2, in flight)
      float res[MB], t0prev[MB], x0o[MB], x0t[MB], x1o[MB], x1t[MB], x2o[MB], x2t[MB];
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        res[m] = 0.f;
        t0prev[m] = 0.f;
        exch(m, tbeg, x0o[m], x0t[m]);
        exch(m, tbeg + 1, x1o[m], x1t[m]);
        exch(m, tbeg + 2, x2o[m], x2t[m]);
        if (PF == 1) heavy(m, tbeg);
      }
      float pn_own = 0.f, pn_t0 = 0.f, ps_own = 0.f, ps_t0 = 0.f;
      if (top) north_of_top(tbeg, pn_own, pn_t0);
      if (ST && bot) south_of_bot(tbeg, ps_own, ps_t0);
      for (int t = tbeg; t < tend; ++t) {
        float qn_own = 0.f, qn_t0 = 0.f, qs_own = 0.f, qs_t0 = 0.f;
        if (top) north_of_top(t + 1, qn_own, qn_t0);
        if (ST && bot) south_of_bot(t + 1, qs_own, qs_t0);
        // Bands in descending order: band m's south neighbours include lane 31
        // of band m-1, whose value must still be the previous step's.
        float dds[MB];
#pragma unroll
        for (int mm = 0; mm < MB; ++mm) {
          const int m = MB - 1 - mm;
          float south = w_below<MB>(res, m, lane), t0s = w_below<MB>(t0prev, m, lane);
          float north = w_above<MB>(x1o, m, lane), t0n = w_above<MB>(x1t, m, lane);
          if (NW > 1 || ST) {
            if (m == 0 && bot) {
              // team: written by warp w-1 at step t-1
              south = ST ? ps_own : xs_val[(t + 1) & 1][T.wid - 1];
              t0s = ST ? ps_t0 : xs_t0[(t + 1) & 1][T.wid - 1];
            }
            if (m == MB - 1 && top) {
              north = pn_own;
              t0n = pn_t0;
            }
          }
          dds[m] = 0.f;
          const int tl = t - R[m].lo;
          if ((unsigned)tl < (unsigned)nx) {
            const int k = R[m].kb + xdir * t;
            const bool frz = (unsigned)(t - R[m].flo) <= (unsigned)flen;
            float nv;
            if (frz) {
              nv = x0o[m];
            } else {
              if (PF == 0) heavy(m, t);
              WFwd o;
              o.own = x0o[m];
              o.t0 = x0t[m];
              o.gx = gx[m];
              o.gy = gy[m];
              o.pa = pa[m];
              o.dsx = dsx[m];
              o.dsy = dsy[m];
              nv = wf_visit(o, res[m], x1o[m], south, north, t0prev[m], x1t[m], t0s, t0n, tl > 0,
                            R[m].hass, tl < nx - 1, R[m].hasn, xdir, ydir, idx, idy);
            }
            if constexpr (PAIR)
              reinterpret_cast<float*>(V.TT)[2 * (size_t)k + 1] = nv;
            else
              V.tau[k] = nv;
            if (s == 0) V.old[k] = x0o[m];
            if (last && !frz) dds[m] = fabsf(nv - old[m]) * x0t[m];
            res[m] = nv;
            t0prev[m] = x0t[m];
          }
          if (NW > 1 && m == MB - 1 && top) {
            xs_val[t & 1][T.wid] = res[m];
            xs_t0[t & 1][T.wid] = t0prev[m];
          }
          // the band's cell constants of the next step, into the registers
          // its visit has just consumed
          if (PF == 1) heavy(m, t + 1);
        }
#pragma unroll
        for (int m = 0; m < MB; ++m) {
          x0o[m] = x1o[m];
          x0t[m] = x1t[m];
          x1o[m] = x2o[m];
          x1t[m] = x2t[m];
          exch(m, t + 3, x2o[m], x2t[m]);
        }
        if (last) {
          // in band order (the order of the row-major visit of a lane)
#pragma unroll
          for (int m = 0; m < MB; ++m) {
            l1 += dds[m];
            lmax = fmaxf(lmax, dds[m]);
          }
        }
        pn_own = qn_own;
        pn_t0 = qn_t0;
        ps_own = qs_own;
        ps_t0 = qs_t0;
        tsync<NW>();
      }
      if (ST && last) w_strip_add(l1acc, l1);
     }
    }
    // FP64 decision over the lanes' partial sums (:1091-1115)
    double sl1, smax = (double)lmax, unused = 0.0;
    if (ST) {
      sl1 = l1acc;
      smax = w_warp_max(smax);
    } else {
      sl1 = (double)l1;
      tsum_max2<NW>(sl1, smax, unused);
    }
    sl1 = sl1 / (double)nx / (double)ny;
    if (fabs(sl1) < TOL_UW && smax < TOL_UW) {
      status = ST_OK;
      break;
    }
  }
  *status_out = status;
  *iters_out = iter > it1 ? it1 : iter;
}

// ---------------------------------------------------------------------------
// adjoint
// ---------------------------------------------------------------------------
// Weights of Ta = src + ww*Ta_W + we*Ta_E + ws*Ta_S + wn*Ta_N (face fluxes of
// :1348-1370 with T = tau*T0 in FP32) and 1/d per interior cell.
template <int NW, bool PAIR>
__device__ inline void w_adj_setup(const PeriodDev& P, const WSlot& V, const Tm<NW>& TM) {
  const int nx = P.nx, ny = P.ny, lane = TM.lane;
  const float idx = (float)(1.0 / P.dx), idy = (float)(1.0 / P.dy);
  const float2* TT = V.TT;  // paired: {T0, tau}
  const float* T0 = V.T0;   // separate
  const float4* PA = P.p4a;
  // T = tau*T0 rounded on its own (no contraction with the differences below)
  auto T = [&](size_t k) {
    if constexpr (PAIR) {
      const float2 q = TT[k];
      return __fmul_rn(q.y, q.x);
    } else {
      return __fmul_rn(V.tau[k], T0[k]);
    }
  };
  for (int j = TM.wid; j < ny; j += NW) {  // rows by warp, columns by lane
    for (int i = lane; i < nx; i += 32) {
      const size_t k = i + (size_t)nx * j;
      if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1) {
        V.W[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        V.id[k] = 0.f;
        continue;
      }
      const size_t w = k - 1, e = k + 1, s = k - nx, n = k + nx;
      const float4 pk = PA[2 * k], pw = PA[2 * w], pe = PA[2 * e], ps = PA[2 * s], pn = PA[2 * n];
      const float Tk = T(k), Tw = T(w), Te = T(e), Ts = T(s), Tn = T(n);
      const float Twn = T(w + nx), Tws = T(w - nx), Ten = T(e + nx), Tes = T(e - nx);
      float4 W;
      const float id = adj_weights(Tk, Tw, Te, Ts, Tn, Twn, Tws, Ten, Tes, pk, pw, pe, ps, pn, idx,
                                   idy, &W);
      V.W[k] = W;
      V.id[k] = id;
    }
  }
  tsync<NW>();
}

struct WAdj {
  bool on;
  float own, old, src;
  float4 w;  // ww, we, ws, wn
};

// HEAVY: the weights, source and iteration-start value too (a step ahead of
// the visit); otherwise only the value the lanes exchange.
template <bool HEAVY>
__device__ __forceinline__ void wa_load(WAdj& o, int t, int v, int nu, int nv, int nx, int xdir,
                                        int ydir, const WSlot& V, const float* fld,
                                        const float* fold, const float* src, bool last) {
  const int u = t - v;
  o.on = v < nv && u >= 0 && u < nu;
  if (!o.on) {
    o.own = 0.f;
    return;
  }
  const int i = xdir > 0 ? 1 + u : nu - u;  // interior [1, nx-2]
  const int j = ydir > 0 ? 1 + v : nv - v;
  const int k = i + nx * j;
  o.own = fld[k];
  if (HEAVY) {
    o.w = V.W[k];
    o.src = src[k];
    if (last) o.old = fold[k];
  }
}

// Buffer holding an adjoint field after `iters` iterations of w_adj_sweeps.
__device__ __forceinline__ float* w_adj_result(float* fld, float* fold, int iters) {
  return (iters & 1) ? fold : fld;
}

// Storage of adjoint field f during the adjoint, in forward state that is
// dead once the adjoint weights are set, so that a solve's two fields can
// be swept side by side: paired layout, field 0 and its second buffer in
// TT's 2N floats, field 1 and its second buffer in G's; separate layout,
// field 0 in tau / old, field 1 in G's 2N floats.
template <bool PAIR>
__device__ __forceinline__ float* w_field(const WSlot& V, int f, size_t N) {
  if constexpr (PAIR) return V.R + (f ? 2 * N : 0);
  return f ? reinterpret_cast<float*>(V.G) : V.tau;
}
template <bool PAIR>
__device__ __forceinline__ float* w_field_old(const WSlot& V, int f, size_t N) {
  if constexpr (PAIR) return V.R + (f ? 3 * N : N);
  return f ? reinterpret_cast<float*>(V.G) + N : V.old;
}

// Sweeps one adjoint field (held in fld, iteration-start values in fold) to
// convergence: the reference's
// absolute rule (:1429) or no change beyond the FP32 resolution of the field.
// Neighbours outside the interior are the boundary's zeros.
//
// D is the depth of the operand ring: at step t the operands of step
// t + D - 1 are loaded.  A visit is four FMAs, so a step is far shorter than
// the latency of its operands (the weights are read once per sweep and do
// not stay in L1); the step loop is unrolled by D so that every ring slot is
// a fixed set of registers and no operand is ever copied.  The solve kernel
// affords D = 2 for a single warp (its forward sweeps hold the register
// file: deeper rings spill) and D = 3 for teams.
//
// Iterations it0 .. it1 (the field is initialised when it0 == 1; a later
// range resumes from where the previous one left it): ST_OK and the
// iteration that converged, or ST_NOT_CONVERGED and it1.  The two buffers
// alternate: iteration i starts from fld (i odd) or fold (i even), its
// first sweep writes the other, which the other three sweeps update in
// place, so the start values stay for the convergence test without a store
// of their own; after iteration i the field is in fold (i odd) or fld (i
// even) -- w_adj_result.
template <int MB, int NW, int D, bool ST>
__device__ inline void w_adj_sweeps(const PeriodDev& P, const WSlot& V, float* fld, float* fold,
                                    const float* src, const Tm<NW>& T, int it0, int it1,
                                    int* status_out, int* iters_out) {
  static_assert(!ST || NW == 1, "strips are swept by one warp");
  const int nx = P.nx, ny = P.ny, lane = T.lane;
  const int nu = nx - 2, nv = ny - 2;
  const int nsteps = nu + nv - 1;
  if (it0 == 1) {
    for (int j = T.wid; j < ny; j += NW)
      for (int i = lane; i < nx; i += 32) {
        const bool in = i > 0 && i < nx - 1 && j > 0 && j < ny - 1;
        fld[i + (size_t)nx * j] = in ? 100.f : 0.f;
        fold[i + (size_t)nx * j] = 0.f;
      }
    tsync<NW>();
  }
  // Teams: as in the forward sweeps, the first row's south value comes
  // through a shared slot from the warp below, the last row's north value
  // from memory a step ahead.  Strips (ST): as in the forward sweeps, both
  // from memory a step ahead.
  const int nstrip = ST ? (nv + 32 * MB - 1) / (32 * MB) : 1;
  __shared__ float xs_val[2][NW > 1 ? NW : 1];
  int iter, status = ST_NOT_CONVERGED;
  for (iter = it0; iter <= it1; ++iter) {
    float l1 = 0.f, lmax = 0.f, vmax = 0.f;
    // iteration start values in xs (read by the first sweep, kept for the
    // convergence test), the sweeps' field in ys: odd iterations start in
    // fld, even ones in fold
    float* const xs = (iter & 1) ? fld : fold;
    float* const ys = (iter & 1) ? fold : fld;
    double l1acc = 0.0;  // strips, last sweep: the strips' reduced sums so far
    for (int s = 0; s < 4; ++s) {
      int xdir, ydir;
      sweep_dirs(s, xdir, ydir);
      const bool last = s == 3;
      const float* const rd = s == 0 ? xs : ys;
     for (int sp = 0; sp < nstrip; ++sp) {
      const int vb = 32 * MB * (ST ? sp : T.wid);
      const int vtop = vb + 32 * MB - 1;
      const bool top = (NW > 1 || ST) && lane == 31 && (ST ? vtop + 1 < nv : T.wid < NW - 1);
      const bool bot = (NW > 1 || ST) && lane == 0 && (ST ? sp > 0 : T.wid > 0);
      const int tbeg = ST ? vb : 0;
      const int tend = ST ? min(vtop, nv - 1) + nu : nsteps;
      if (ST) l1 = 0.f;
      auto north_of_top = [&](int tau) {
        const int u = tau - vtop;
        if (u < 0 || u >= nu || vtop + 1 >= nv) return 0.f;
        return rd[(xdir > 0 ? 1 + u : nu - u) + nx * (ydir > 0 ? 2 + vtop : nv - 1 - vtop)];
      };
      // strips: the new value south of the bottom row at step tau (the strip
      // below wrote it in this sweep: the buffer the sweep writes)
      auto south_of_bot = [&](int tau) {
        const int u = tau - vb;
        if (u < 0 || u >= nu || vb < 1) return 0.f;
        return ys[(xdir > 0 ? 1 + u : nu - u) + nx * (ydir > 0 ? vb : nv + 1 - vb)];
      };
      // A cell is written only at its own visit and the weights, sources and
      // iteration-start values are fixed within a sweep, so operands loaded
      // D - 1 steps early are the values a load at the visit would see.
      float res[MB];
      WAdj ring[D][MB];
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        res[m] = 0.f;
#pragma unroll
        for (int d = 0; d < D; ++d)
          wa_load<true>(ring[d][m], tbeg + d, vb + lane + 32 * m, nu, nv, nx, xdir, ydir, V, rd,
                        xs, src, last);
      }
      float pn = top ? north_of_top(tbeg) : 0.f;
      float ps = (ST && bot) ? south_of_bot(tbeg) : 0.f;
      for (int t0 = tbeg; t0 < tend; t0 += D) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const int t = t0 + d;
          if (t >= tend) break;  // the same for every thread of the team
          WAdj(&cur)[MB] = ring[d];
          const WAdj(&nxt)[MB] = ring[(d + 1) % D];
          const float qn = top ? north_of_top(t + 1) : 0.f;
          const float qs = (ST && bot) ? south_of_bot(t + 1) : 0.f;
          float south[MB], north[MB], nown[MB];
#pragma unroll
          for (int m = 0; m < MB; ++m) nown[m] = nxt[m].own;
          w_from_below<MB>(res, south, lane);
          w_from_above<MB>(nown, north, lane);
          if (NW > 1 || ST) {
            // team: written by warp w-1 at step t-1
            if (bot) south[0] = ST ? ps : xs_val[(t + 1) & 1][T.wid - 1];
            if (top) north[MB - 1] = pn;
          }
#pragma unroll
          for (int m = 0; m < MB; ++m) {
            if (cur[m].on) {
              const int v = vb + lane + 32 * m, u = t - v;
              const int k = (xdir > 0 ? 1 + u : nu - u) + nx * (ydir > 0 ? 1 + v : nv - v);
              const float west = u > 0 ? res[m] : 0.f;
              const float east = u < nu - 1 ? nown[m] : 0.f;
              const float sth = v > 0 ? south[m] : 0.f;
              const float nth = v < nv - 1 ? north[m] : 0.f;
              const float tw = xdir > 0 ? west : east, te = xdir > 0 ? east : west;
              const float ts = ydir > 0 ? sth : nth, tn = ydir > 0 ? nth : sth;
              const float val = adj_update(cur[m].src, cur[m].w, tw, te, ts, tn);
              ys[k] = val;
              if (last) {
                const float dd = fabsf(val - cur[m].old);
                l1 += dd;
                lmax = fmaxf(lmax, dd);
                vmax = fmaxf(vmax, fabsf(val));
              }
              res[m] = val;
            }
          }
          // this slot now takes the operands of step t + D
#pragma unroll
          for (int m = 0; m < MB; ++m)
            wa_load<true>(ring[d][m], t + D, vb + lane + 32 * m, nu, nv, nx, xdir, ydir, V, rd,
                          xs, src, last);
          if (NW > 1 && top) xs_val[t & 1][T.wid] = res[MB - 1];
          pn = qn;
          ps = qs;
          tsync<NW>();
        }
      }
      if (ST && last) w_strip_add(l1acc, l1);
     }
    }
    double sl1, smax = (double)lmax, svmax = (double)vmax;
    if (ST) {
      sl1 = l1acc;
      smax = w_warp_max(smax);
      svmax = w_warp_max(svmax);
    } else {
      sl1 = (double)l1;
      tsum_max2<NW>(sl1, smax, svmax);
    }
    sl1 = sl1 / (double)(nx * ny);
    if ((fabs(sl1) < TOL_JSE && smax < TOL_JSE) || smax <= svmax * 0x1p-21) {
      status = ST_OK;
      break;
    }
  }
  *status_out = status;
  *iters_out = iter > it1 ? it1 : iter;
}

// T = tau*T0 at a node (FP64 product of the FP32 factors)
template <bool PAIR>
__device__ __forceinline__ double w_T(const WSlot& V, size_t k) {
  const float2 q = w_t0tau<PAIR>(V, k);
  return (double)q.y * (double)q.x;
}

// interp2_0_dp on the caller's increasing degree grid (src/shared/utils.f90:917-942)
template <bool PAIR>
__device__ inline bool w_interp(const PeriodDev& P, const WSlot& V, double xq, double yq,
                                double* out) {
  const int nx = P.nx, ny = P.ny;
  int lo = -1, hi = nx;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (xq >= P.xdeg[mid]) lo = mid; else hi = mid;
  }
  if (lo < 0 || lo >= nx - 1) return false;
  int ylo = -1, yhi = ny;
  while (yhi - ylo > 1) {
    const int mid = (ylo + yhi) >> 1;
    if (yq >= P.ydeg[mid]) ylo = mid; else yhi = mid;
  }
  if (ylo < 0 || ylo >= ny - 1) return false;
  const double* x = P.xdeg;
  const double* y = P.ydeg;
  const int x1 = lo, x2 = lo + 1, y1 = ylo, y2 = ylo + 1;
  const double vn = fabs((x[x2] - x[x1]) * (y[y2] - y[y1]));
  const double n1 = fabs((x[x2] - xq) * (y[y2] - yq));
  const double n2 = fabs((x[x1] - xq) * (y[y2] - yq));
  const double n3 = fabs((x[x2] - xq) * (y[y1] - yq));
  const double n4 = fabs((x[x1] - xq) * (y[y1] - yq));
  double r = 0;
  r = r + w_T<PAIR>(V, x1 + (size_t)nx * y1) * (n1 / vn);
  r = r + w_T<PAIR>(V, x2 + (size_t)nx * y1) * (n2 / vn);
  r = r + w_T<PAIR>(V, x1 + (size_t)nx * y2) * (n3 / vn);
  r = r + w_T<PAIR>(V, x2 + (size_t)nx * y2) * (n4 / vn);
  *out = r;
  return true;
}

// ---------------------------------------------------------------------------
// the tail of a solve
// ---------------------------------------------------------------------------
// Receiver times, misfit, outlier weights (src/measadj.f90:71-72, 82-84);
// returns the status (ST_BAD_ARG for a receiver outside the grid).
template <int NW, bool PAIR>
__device__ inline int w_receivers(const BatchArgs& A, const PeriodDev& P, const WSlot& V, int s,
                                  int r0, int nr, const Tm<NW>& T, int st) {
  int bad = 0;
  for (int r = T.tid; r < nr; r += 32 * NW) {
    double v = 0.0;
    if (!w_interp<PAIR>(P, V, A.recx[r0 + r], A.recy[r0 + r], &v)) bad = 1;
    A.tekio[r0 + r] = v;
    A.tt_fwd[A.path[r0 + r]] = v;
  }
  if (NW == 1) bad = __any_sync(FULL, bad);
  else bad = __syncthreads_or(bad);
  if (A.Tout) {
    const size_t N = (size_t)P.nx * P.ny;
    for (size_t k = T.tid; k < N; k += 32 * NW) A.Tout[A.kslot[s] + k] = w_T<PAIR>(V, k);
  }
  tsync<NW>();
  if (T.tid == 0) {
    double ssum = 0;
    for (int r = 0; r < nr; ++r) {
      const double d = A.tekio[r0 + r] - A.tt[r0 + r];
      ssum = ssum + A.weight[r0 + r] * (d * d);
    }
    A.chi[s] = 0.5 * ssum;
    for (int r = 0; r < nr; ++r) {
      double wt = A.weight[r0 + r];
      if (fabs(A.tekio[r0 + r] - A.tt[r0 + r]) / A.tt[r0 + r] > 0.5) wt = 0.;
      A.wgt_eff[r0 + r] = wt;
    }
  }
  tsync<NW>();
  return (bad && st == ST_OK) ? ST_BAD_ARG : st;
}

// Adjoint coefficients and the scaled sources of nf fields: weight*(tekio-tt)
// (src/measadj.f90:88) and -weight (:102), splat bilinearly over the cell
// area (src/eikon_solver_2d.f90:1328-1336) and scaled by 1/d.
template <int NW, bool PAIR>
__device__ inline int w_adj_sources(const BatchArgs& A, const PeriodDev& P, const WSlot& V,
                                    int r0, int nr, int nf, const Tm<NW>& T, int st) {
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  w_adj_setup<NW, PAIR>(P, V, T);
  // (the fields' arrays picked by selects: an indexed V.src[f] would put
  // the whole slot descriptor in local memory)
  for (int f = 0; f < nf; ++f) {
    float* const sf = f ? V.src[1] : V.src[0];
    for (size_t k = T.tid; k < N; k += 32 * NW) sf[k] = 0.f;
  }
  tsync<NW>();
  if (T.wid == 0)
    st = adj_sources_warp(A, P, r0, nr, nf, V.src[0], nf == 2 ? V.src[1] : V.src[0], V.id,
                          [nx](int i, int j) { return i + nx * j; }, T.lane, st);
  st = tbcast<NW>(st);
  tsync<NW>();
  return st;
}

// Mask (src/eikon_solver_2d.f90:1449-1467) and the kernel slot adj/svel**k
// (src/acqui.f90:314-315) of adjoint field f, FP32 here, summed per period
// in FP64.
template <int NW>
__device__ inline void w_slot(const BatchArgs& A, const PeriodDev& P, const float* field,
                              const WSolve& w, int s, int f, const Tm<NW>& T) {
  const int nx = P.nx, ny = P.ny, lane = T.lane;
  float* out = reinterpret_cast<float*>(f == 0 ? A.kcontrib : A.kcontrib_den) + A.kslot[s];
  // groups of G cells: loads first, then stores (as in w_adj_setup)
  constexpr int G = 4;
  for (int j = T.wid; j < ny; j += NW)  // rows by warp
    for (int i0 = lane; i0 < nx; i0 += 32 * G) {
      float isv[G], ta[G];
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const int i = i0 + 32 * g;
        isv[g] = 0.f;
        ta[g] = 0.f;
        if (i < nx) {
          const size_t k = i + (size_t)nx * j;
          const float4 pb = P.p4b[2 * k];
          isv[g] = A.mode == 3 ? pb.w : pb.z;
          ta[g] = field[k];
        }
      }
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const int i = i0 + 32 * g;
        if (i < nx) out[i + (size_t)nx * j] = w.mbox.has(i, j) ? 0.f : ta[g] * isv[g];
      }
    }
  tsync<NW>();
}

// ---------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------
// One warp per block; MINW resident warps per SM is the launch bound.  The
// register file is split between the SM's four schedulers, so 8 warps (two
// per scheduler) allow 255 registers a thread and 12 warps (three) 168.
//
// Work items.  With A.items == 1 a warp takes whole solves.  With A.items > 1
// each solve is cut into items -- A.fwd_items consecutive forward items of
// kSplitIter iterations each (the first also computes T0, the last runs to
// convergence and adds receivers, misfit, adjoint coefficients and
// sources), then A.adj_parts items per adjoint field (iteration ranges of
// kAdjSplitIter, the last to convergence, then the field's kernel slot) --
// each solve has its own workspace slot and state record.  The queue hands
// out every solve's forward item 0, then every item 1, and so on, so that
// the last round of a batch is a short item rather than a whole solve, then
// every solve's first part of each field (a solve's two fields next to each
// other, so that two warps sweep them side by side; field 1 lives in the T0
// gradient's array, dead by then), then every second part, and so on.  A
// forward item waits (bounded) for the previous item of its solve, a
// field's first part for the last forward item, a later part for the
// field's previous part; each was taken earlier by a resident warp, so the
// waits cannot form a cycle.  A part records the field's iterations and
// status; the part that finishes a field (it converged, or it is the last)
// writes the kernel slot and counts the field, and the one that finishes a
// solve's last field reports the solve (its fields' statuses taken in field
// order); parts after convergence only mark themselves done.
// (measured on the 1280-solve, 120 x 120 evaluation: forward items of one
// iteration, five of them, and three parts per adjoint field, 17.6 ms,
// against 18.0 with three forward items of two iterations)
constexpr int kSplitIter = 1;
constexpr int kFwdItems = 5;
// adjoint iterations per part of a field cut into A.adj_parts items (the
// last part runs to convergence)
constexpr int kAdjSplitIter = 1;
constexpr int kAdjParts = 3;

// Items per solve for `mode` when solves are cut.
__host__ __device__ inline int w_items_for_mode(int mode, int fwd_items = kFwdItems) {
  return fwd_items + (mode == 3 ? 2 : (mode == 2 ? 1 : 0));
}

template <int MB, int PF, int MINW, int NW, bool ST>
__global__ void __launch_bounds__(32 * NW, MINW / NW) k_batch_fp32w(BatchArgs A) {
  // workspace layout: paired forward state for strips and teams, separate
  // for the one-warp kernel (batch_fp32w_ws_doubles)
  constexpr bool kPair = ST || NW > 1;
  const Tm<NW> T = this_team<NW>();
  const int lane = T.lane;
  const bool cut = A.items > 1;
  const int nitem = cut ? A.items : 1;
  float* kf = reinterpret_cast<float*>(A.kcontrib);
  float* kdf = reinterpret_cast<float*>(A.kcontrib_den);
  const int nf = A.mode == 3 ? 2 : 1;
  const int nfwd = cut && A.fwd_items > 0 ? A.fwd_items : kFwdItems;   // forward items
  const int nparts = cut && A.adj_parts > 0 ? A.adj_parts : 1;         // items per field
  for (;;) {
    int q = 0;
    if (T.tid == 0) q = atomicAdd(A.queue, 1);
    q = tbcast<NW>(q);
    if (q >= A.nsolve * nitem) break;
    // queue order: every solve's forward item 0, then every item 1, ...;
    // then every solve's first part of each adjoint field (a solve's fields
    // next to each other), then every second part, ...
    int item = q / A.nsolve, si = q % A.nsolve, part = 0, fi = 0;
    if (cut && item >= nfwd) {
      const int r = q - nfwd * A.nsolve;
      part = r / (A.nsolve * nf);
      si = (r % (A.nsolve * nf)) / nf;
      fi = r % nf;
      item = nfwd + part * nf + fi;
    }
    const int s = A.order[si];
    int* const ss = cut ? A.sstate + (size_t)kSolveStateInts * s : nullptr;
    if (cut && item == 0 && s == A.hold_solve) continue;  // test hook: never done
    if (cut && item > 0) {
      // a forward item: the previous forward item of this solve; an adjoint
      // field's first part: the whole forward; a later part: the field's
      // previous part (each taken earlier by a resident warp)
      const bool onfield = item >= nfwd && part > 0;
      const int need = item < nfwd ? item : (part == 0 ? nfwd : part);
      const int limit =
          (s == A.hold_solve && A.item_wait_limit > 0) ? A.item_wait_limit : kItemWaitLimit;
      int d = ld_acquire(ss + SS_DONE), it = 0;
      int g = onfield ? ld_acquire(ss + (fi ? SS_AD1 : SS_AD0)) : d;
      while (d >= 0 && g < need && it < limit) {
        __nanosleep(128);
        d = ld_acquire(ss + SS_DONE);
        g = onfield ? ld_acquire(ss + (fi ? SS_AD1 : SS_AD0)) : d;
        ++it;
      }
      // every thread acquired the state itself; the team takes one decision
      bool failed = d < 0, late = d >= 0 && g < need;
      if (NW > 1) {
        failed = __syncthreads_or(failed);
        late = !failed && __syncthreads_or(late);
      }
      if (failed) continue;  // the solve failed in an earlier item
      if (late) {            // wait limit: report and drop the solve
        // the solve contributes nothing (as a solve whose source is on the
        // boundary): zero receiver times, misfit and kernel slots
        const PeriodDev& Pz = A.periods[A.pidx[s]];
        const size_t Nz = (size_t)Pz.nx * Pz.ny;
        const int rz = A.rec_off[s], nz = A.nrec[s];
        for (int r = T.tid; r < nz; r += 32 * NW) {
          A.tekio[rz + r] = 0.0;
          A.wgt_eff[rz + r] = 0.0;
          A.tt_fwd[A.path[rz + r]] = 0.0;
        }
        if (A.mode >= 2)
          for (size_t kk = T.tid; kk < Nz; kk += 32 * NW) {
            kf[A.kslot[s] + kk] = 0.f;
            if (A.mode == 3) kdf[A.kslot[s] + kk] = 0.f;
          }
        if (A.Tout)
          for (size_t kk = T.tid; kk < Nz; kk += 32 * NW) A.Tout[A.kslot[s] + kk] = 0.0;
        __threadfence();
        tsync<NW>();
        if (T.tid == 0) {
          A.chi[s] = 0.0;
          A.status[s] = ST_TIMEOUT;
          A.fwd_iters[s] = 0;
          A.adj_iters[s] = 0;
          if (A.fwd_updates) A.fwd_updates[s] = 0;
          st_release(ss + SS_DONE, -1);
        }
        tsync<NW>();
        continue;
      }
    }
    const PeriodDev P = A.periods[A.pidx[s]];
    const int nx = P.nx, ny = P.ny;
    const size_t N = (size_t)nx * ny;
    const int r0 = A.rec_off[s], nr = A.nrec[s];
    const WSlot V = wcarve(A.ws + (cut ? (long long)s : (long long)blockIdx.x) * A.ws_doubles, N,
                           kPair);
    const double xd0 = A.srcx[s], yd0 = A.srcy[s];
    const double x0 = xd0 / 180.0 * PI_S, y0 = yd0 / 180.0 * PI_S;
    unsigned long long* const pc = A.phase_cycles;
    long long c0 = pc ? clock64() : 0;
    // adds the cycles since the previous mark to phase `ph` (lane 0, when on)
    auto mark = [&](int ph) {
      if (pc) {
        const long long c1 = clock64();
        if (T.tid == 0) atomicAdd(pc + ph, (unsigned long long)(c1 - c0));
        c0 = c1;
      }
    };
    // this warp's writes of the item become visible, then the item is done
    auto finish_item = [&](int done) {
      if (cut) {
        __threadfence();
        tsync<NW>();
        if (T.tid == 0) st_release(ss + SS_DONE, done);
      }
      tsync<NW>();
    };
    const WSolve w = w_locate(P, x0, y0, xd0, yd0, lane);
    const int nitems_mode = w_items_for_mode(A.mode, nfwd);
    const int first = cut ? item : 0;                 // first item done here
    const int lastit = cut ? item : nitems_mode - 1;  // last item done here
    int fst = ST_OK, fit = 0, st = ST_OK, its0 = 0, its1 = 0, ast0 = ST_OK, ast1 = ST_OK;
    if (cut && first > 0) {
      int v0 = 0, v1 = 0, v2 = 0;
      if (T.tid == 0) {
        v0 = ss[SS_FIT];
        v1 = ss[SS_FST];
        v2 = ss[SS_ST];
      }
      fit = tbcast<NW>(v0);
      fst = tbcast<NW>(v1);
      st = tbcast<NW>(v2);
    }
    if (first == 0 && w.status != ST_OK) {
      for (int r = T.tid; r < nr; r += 32 * NW) {
        A.tekio[r0 + r] = 0.0;
        A.wgt_eff[r0 + r] = 0.0;
        A.tt_fwd[A.path[r0 + r]] = 0.0;
      }
      if (A.mode >= 2)
        for (size_t kk = T.tid; kk < N; kk += 32 * NW) {
          kf[A.kslot[s] + kk] = 0.f;
          if (A.mode == 3) kdf[A.kslot[s] + kk] = 0.f;
        }
      if (A.Tout)
        for (size_t kk = T.tid; kk < N; kk += 32 * NW) A.Tout[A.kslot[s] + kk] = 0.0;
      if (T.tid == 0) {
        A.chi[s] = 0.0;
        A.status[s] = w.status;
        A.fwd_iters[s] = 0;
        A.adj_iters[s] = 0;
        if (A.fwd_updates) A.fwd_updates[s] = 0;
      }
      finish_item(-1);
      continue;
    }
    // forward sweeps: forward item k runs iterations k*kSplitIter+1 ..
    // (k+1)*kSplitIter, the last one (a whole solve: all) up to MaxIter,
    // unless an earlier item converged
    if (first == 0) {
      w_t0<NW, kPair>(P, x0, y0, w, V, T);
      mark(PH_SETUP);
    }
    if (first < nfwd && (first == 0 || (fst != ST_OK && fit < MAXITER_UW))) {
      const int it0 = first == 0 ? 1 : fit + 1;
      const int it1 = (cut && first < nfwd - 1) ? (first + 1) * kSplitIter : MAXITER_UW;
      int n = 0;
      w_fwd_sweeps<MB, PF, NW, ST>(P, V, w, T, it0, it1, &fst, &n);
      fit = n;
      mark(PH_FWD);
    }
    if (cut && first < nfwd - 1) {
      if (T.tid == 0) {
        ss[SS_FIT] = fit;
        ss[SS_FST] = fst;
      }
      finish_item(first + 1);
      continue;
    }
    if (first <= nfwd - 1) {
      if (A.fwd_updates && T.tid == 0) {
        const double frozen = (double)(w.box.i1 - w.box.i0 + 1) * (w.box.j1 - w.box.j0 + 1);
        A.fwd_updates[s] = (double)fit * 4.0 * ((double)N - frozen);
      }
      st = w_receivers<NW, kPair>(A, P, V, s, r0, nr, T, fst);
      mark(PH_RECV);
      if (A.mode >= 2) {
        st = w_adj_sources<NW, kPair>(A, P, V, r0, nr, nf, T, st);
        mark(PH_ADJ_SETUP);
      }
      if (cut && A.mode >= 2) {
        if (T.tid == 0) {
          ss[SS_FIT] = fit;
          ss[SS_ST] = st;
        }
        finish_item(nfwd);
        continue;
      }
    }
    // adjoint field(s) f0 .. f1 (an adjoint item: one part of one field)
    const int f0 = cut ? fi : 0;
    const int f1 = A.mode >= 2 ? (cut ? fi : nf - 1) : -1;
    bool field_done = true;
    for (int f = f0; f <= f1; ++f) {
      int ast = ST_OK, n = 0, it0 = 1, it1 = MAXITER_JSE;
      if (cut && part > 0) {
        // this field's earlier parts: converged (nothing left) or not
        int v0 = 0, v1 = 0;
        if (T.tid == 0) {
          v0 = ss[f ? SS_ITS1 : SS_ITS0];
          v1 = ss[f ? SS_AST1 : SS_AST0];
        }
        n = tbcast<NW>(v0);
        ast = tbcast<NW>(v1);
        it0 = n + 1;
      }
      if (cut && part < nparts - 1) it1 = (part + 1) * kAdjSplitIter;
      float* const fld = f ? w_field<kPair>(V, 1, N) : w_field<kPair>(V, 0, N);
      float* const fold = f ? w_field_old<kPair>(V, 1, N) : w_field_old<kPair>(V, 0, N);
      const bool earlier = cut && part > 0 && ast == ST_OK;  // converged in an earlier part
      if (!earlier) {
        w_adj_sweeps<MB, NW, (PF == 1 && NW > 1) ? 3 : 2, ST>(
            P, V, fld, fold, f ? V.src[1] : V.src[0], T, it0, it1, &ast, &n);
        mark(PH_ADJ);
      }
      if (f == 0) { its0 = n; ast0 = ast; } else { its1 = n; ast1 = ast; }
      field_done = !earlier && (ast == ST_OK || !cut || part == nparts - 1);
      if (field_done) {
        w_slot<NW>(A, P, w_adj_result(fld, fold, n), w, s, f, T);
        mark(PH_SLOT);
      }
    }
    if (cut && f1 >= 0) {
      // one part of one field: the field's iterations and status into the
      // solve's record, then the part is done; the part that finishes the
      // field counts it, and the one that finishes the solve's last field
      // reports the solve
      if (T.tid == 0) {
        ss[f0 ? SS_ITS1 : SS_ITS0] = f0 ? its1 : its0;
        ss[f0 ? SS_AST1 : SS_AST0] = f0 ? ast1 : ast0;
      }
      __threadfence();
      tsync<NW>();
      if (T.tid == 0) st_release(ss + (f0 ? SS_AD1 : SS_AD0), part + 1);
      if (!field_done) {
        tsync<NW>();
        continue;
      }
      int nprev = 0;
      if (T.tid == 0) nprev = atomicAdd(ss + SS_ADJ, 1);
      nprev = tbcast<NW>(nprev);
      if (nprev < nf - 1) {
        tsync<NW>();
        continue;
      }
      __threadfence();
      int v0 = 0, v1 = 0, v2 = 0, v3 = 0;
      if (T.tid == 0) {
        v0 = ld_acquire(ss + SS_ITS0);
        v1 = ld_acquire(ss + SS_AST0);
        v2 = nf > 1 ? ld_acquire(ss + SS_ITS1) : 0;
        v3 = nf > 1 ? ld_acquire(ss + SS_AST1) : ST_OK;
      }
      its0 = tbcast<NW>(v0);
      ast0 = tbcast<NW>(v1);
      its1 = tbcast<NW>(v2);
      ast1 = tbcast<NW>(v3);
    }
    // field statuses in field order, as one warp sweeping them in turn
    if (A.mode >= 2 && ast0 != ST_OK && st == ST_OK) st = ast0;
    if (A.mode == 3 && ast1 != ST_OK && st == ST_OK) st = ast1;
    // the solve's last item: its outputs
    if (T.tid == 0) {
      A.status[s] = st;
      A.fwd_iters[s] = fit;
      A.adj_iters[s] = its0 > its1 ? its0 : its1;
      if (A.adj_updates && A.mode >= 2)
        A.adj_updates[s] = (double)(its0 + its1) * 4.0 * (nx - 2) * (ny - 2);
    }
    finish_item(nitems_mode);
  }
}

int fp32w_bands(int max_ny) { return (max_ny + 31) / 32; }

// Variants of the warp kernel: operand loads, resident warps per SM, whole
// solves or solves cut into items, teams or strips above 128 rows.
//   0: every operand loaded a step ahead into registers, 8 warps per SM, items
//   1: the same, whole solves
//   2: cell constants loaded at the visit, 12 warps per SM, items
//   3: cell constants loaded at the visit, 8 warps per SM, whole solves
//   4: grids of more than 128 rows swept in strips by one warp; items (their
//      forward whole, one resident warp per solve)
//   5: the same strips, whole solves
// On grids of at most 128 rows variants 4 and 5 are variants 0 and 1.
constexpr int kFp32wVariants = 6;
int fp32w_variant_count() { return kFp32wVariants; }
bool fp32w_variant_items(int variant) { return variant == 0 || variant == 2 || variant == 4; }
bool fp32w_variant_strips(int variant) { return variant >= 4; }
int fp32w_items_for_mode(int mode) { return w_items_for_mode(mode); }
int fp32w_fwd_items(int variant, int bands) {
  return fp32w_variant_strips(variant) && bands > 4 ? 1 : kFwdItems;
}
int fp32w_adj_parts(int variant) { return fp32w_variant_items(variant) ? kAdjParts : 1; }

template <int MB, int PF, int MINW, int NW, bool ST>
static void launch_w(const BatchArgs& a, int grid, cudaStream_t st) {
  k_batch_fp32w<MB, PF, MINW, NW, ST><<<grid, 32 * NW, 0, st>>>(a);
}

template <int MB, int PF, int MINW, int NW, bool ST>
static int occupancy_w() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_fp32w<MB, PF, MINW, NW, ST>, 32 * NW,
                                                0);
  return n;
}

template <int MB, int NW>
static void launch_mb(const BatchArgs& a, int grid, int variant, cudaStream_t st) {
  switch (variant) {
    case 0:
    case 1:
    case 4:
    case 5: launch_w<MB, 1, 8, NW, false>(a, grid, st); break;
    case 2: launch_w<MB, 0, 12, NW, false>(a, grid, st); break;
    default: launch_w<MB, 0, 8, NW, false>(a, grid, st); break;
  }
}

template <int MB, int NW>
static int occupancy_mb(int variant) {
  switch (variant) {
    case 0:
    case 1:
    case 4:
    case 5: return occupancy_w<MB, 1, 8, NW, false>();
    case 2: return occupancy_w<MB, 0, 12, NW, false>();
    default: return occupancy_w<MB, 0, 8, NW, false>();
  }
}

// Grids of more than 128 rows: teams of fp32w_team(ny) warps of four bands.
int fp32w_team(int max_ny) { return max_ny <= 32 * 4 ? 1 : (max_ny + 127) / 128; }

// Threads per block: a team's warps, or one warp (strips).
int fp32w_block(int bands, int variant) {
  return bands <= 4 || fp32w_variant_strips(variant) ? 32 : 32 * fp32w_team(32 * bands);
}

void launch_batch_fp32w(const BatchArgs& a, int grid, int bands, int variant, cudaStream_t st) {
  switch (bands) {
    case 1: launch_mb<1, 1>(a, grid, variant, st); break;
    case 2: launch_mb<2, 1>(a, grid, variant, st); break;
    case 3: launch_mb<3, 1>(a, grid, variant, st); break;
    case 4: launch_mb<4, 1>(a, grid, variant, st); break;
    default:
      if (fp32w_variant_strips(variant)) {
        launch_w<4, 1, 8, 1, true>(a, grid, st);
        break;
      }
      switch (fp32w_team(32 * bands)) {
        case 2: launch_mb<4, 2>(a, grid, variant, st); break;
        case 3: launch_mb<4, 3>(a, grid, variant, st); break;
        default: launch_mb<4, 4>(a, grid, variant, st); break;
      }
  }
}

int batch_fp32w_max_blocks_per_sm(int bands, int variant) {
  switch (bands) {
    case 1: return occupancy_mb<1, 1>(variant);
    case 2: return occupancy_mb<2, 1>(variant);
    case 3: return occupancy_mb<3, 1>(variant);
    case 4: return occupancy_mb<4, 1>(variant);
    default:
      if (fp32w_variant_strips(variant)) return occupancy_w<4, 1, 8, 1, true>();
      switch (fp32w_team(32 * bands)) {
        case 2: return occupancy_mb<4, 2>(variant);
        case 3: return occupancy_mb<4, 3>(variant);
        default: return occupancy_mb<4, 4>(variant);
      }
  }
}

}  // namespace sgb
