// kernels_fp32d.cu -- FP32-factored batched solve, one warp per (period,
// source) solve, on the diagonal layouts with the wavefront's operands
// staged in shared memory by bulk asynchronous copies (grids of at most 128
// rows).
//
// The wavefront is the one of the row-per-lane kernel: in each of the four
// sweeps lane l owns the logical rows v = l + 32*m (m < MB) and at step t
// visits the cell u = t - v of each of its rows, which reproduces the
// reference's in-place Gauss-Seidel order; west / south neighbours come from
// registers and __shfl_up, east / north (not yet updated) from the next
// step's operands.  The cells of a step form one anti-diagonal of the
// sweep's frame, and every per-cell array is stored by diagonals (common.cuh
// diag_index): the sweeps x+y+ and x-y- run along i + j = const (family 0),
// x+y- and x-y+ along i - j = const (family 1), each diagonal contiguous.
// So the operands of a step are a handful of contiguous rows, which one lane
// copies into a ring of NS shared-memory stages (cp.async.bulk with an
// mbarrier per stage) NS steps before they are used; the other lanes wait on
// the stage's barrier and read their elements from shared memory.  Nothing
// of a cell is held in registers across steps except the values the lanes
// exchange, and no load latency is exposed in a step.
//
// Read-only arrays (T0 and its gradient, metric, slowness, adjoint weights
// and sources) are kept in both families; the swept field is transposed
// between them when the sweep order switches family (twice an iteration).
// Precision is that of the row-per-lane kernel: the same visit, T0 and
// adjoint arithmetic, so both give the same bits.
//
// Every wait on a stage is bounded; a stage that does not arrive ends the
// warp's work with SURFATT_TIMEOUT for its solve after the copies still in
// flight have been waited for (bounded as well).
#include "warp_common.cuh"

namespace sgb {

// ---------------------------------------------------------------------------
// workspace
// ---------------------------------------------------------------------------
// Per-solve workspace (floats), D = diag_cells(nx, ny):
//   tau[2]     2D   swept field (forward tau, then each adjoint field)
//   old        D    field at the start of the iteration (family 0)
//   id         D    1/d of the adjoint update (family 0)
//   src[2][2]  4D   scaled adjoint sources, [field][family]
//   t0[2]      2D   T0 per family
//   gxy[2]     4D   {T0x, T0y} per family
//   W[0]       4D   adjoint weights (family 0); W[1] reuses gxy (dead after
//                   the forward sweeps)
//   col        2nx  sin / cos of half the longitude offset per column
long long batch_fp32d_ws_doubles(long long max_dcells, int max_nx) {
  const long long floats = 18 * max_dcells + 2 * (long long)max_nx + 64;
  const long long d = (floats + 1) / 2;
  return (d + 31) / 32 * 32;  // keep every slot 256-byte aligned
}

struct DSlot {
  float* tau[2];
  float* old;
  float* id;
  float* src[2][2];
  float* t0[2];
  float2* gxy[2];
  float4* W[2];
  float* col;
};

__device__ inline DSlot dcarve(double* base, long long D) {
  float* f = reinterpret_cast<float*>(base);
  DSlot V;
  V.tau[0] = f;
  V.tau[1] = f + D;
  V.old = f + 2 * D;
  V.id = f + 3 * D;
  V.src[0][0] = f + 4 * D;
  V.src[0][1] = f + 5 * D;
  V.src[1][0] = f + 6 * D;
  V.src[1][1] = f + 7 * D;
  V.t0[0] = f + 8 * D;
  V.t0[1] = f + 9 * D;
  V.gxy[0] = reinterpret_cast<float2*>(f + 10 * D);
  V.gxy[1] = reinterpret_cast<float2*>(f + 12 * D);
  V.W[0] = reinterpret_cast<float4*>(f + 14 * D);
  V.W[1] = reinterpret_cast<float4*>(f + 10 * D);
  V.col = f + 18 * D;
  return V;
}

// Geometry of one grid in the diagonal layouts.
struct DGeom {
  int nx, ny, pitch, nd;  // nd = nx + ny - 1 diagonals
};

__device__ __forceinline__ int dix(const DGeom& g, int fam, int i, int j) {
  return diag_index(fam, i, j, g.ny, g.pitch);
}

// ---------------------------------------------------------------------------
// stages: bulk copies into shared memory completing on an mbarrier
// ---------------------------------------------------------------------------
// Bytes of one stage per element of a diagonal (the forward's rows: tau 4,
// T0 4, gradient 8, metric 16, one-sided terms 8, iteration-start value 4;
// the adjoint's rows -- tau, sources, weights, old -- reuse the same space).
constexpr int kStageBytesPerElem = 44;
constexpr int kStOffT0 = 4, kStOffGxy = 8, kStOffQa = 16, kStOffQd = 32, kStOffOld = 40;
// Bounded waits on a stage (try_wait rounds, each suspending briefly).
constexpr int kStageWaitLimit = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, unsigned bytes) {
  asm volatile(
      "{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(bar),
      "r"(bytes)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Global -> shared bulk copy (addresses 16-byte aligned, bytes a multiple of 16).
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, unsigned bytes,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

// Generic-proxy global writes of this thread made visible to later bulk copies.
__device__ __forceinline__ void fence_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}
// Generic-proxy shared-memory accesses ordered before later bulk copies.
__device__ __forceinline__ void fence_async_shared() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Bulk prefetch of `bytes` (a multiple of 16) at a 16-byte aligned address into L2.
__device__ __forceinline__ void l2_prefetch(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// The ring of one warp: NS stages of `stage_bytes` each and one mbarrier per
// stage.  Fill number n (counted over the warp's whole life) goes to stage
// n % NS and completes phase (n / NS) & 1 of its barrier.
template <int NS>
struct Ring {
  char* base;
  uint32_t bar0;
  unsigned stage_bytes;
  unsigned long long next;  // fills issued so far (equal in all lanes)
  unsigned long long* wait_cycles;  // optional: cycles spent in wait(), summed

  __device__ char* stage(unsigned long long n) const {
    return base + (size_t)(n % NS) * stage_bytes;
  }
  __device__ uint32_t bar(unsigned long long n) const { return bar0 + 8u * (unsigned)(n % NS); }
  __device__ unsigned parity(unsigned long long n) const { return (unsigned)((n / NS) & 1ull); }
  // all lanes: bounded wait for fill n
  __device__ bool wait(unsigned long long n) const {
    const uint32_t b = bar(n);
    const unsigned ph = parity(n);
    const long long c0 = wait_cycles ? clock64() : 0;
    bool ok = false;
    for (int it = 0; it < kStageWaitLimit && !ok; ++it) ok = mbar_try_wait(b, ph);
    if (wait_cycles && threadIdx.x == 0) atomicAdd(wait_cycles, (unsigned long long)(clock64() - c0));
    return ok;
  }
  // all lanes: after a failed wait, wait (bounded) for fills [from, next)
  __device__ void drain(unsigned long long from) const {
    for (unsigned long long n = from; n < next; ++n) wait(n);
  }
};

// ---------------------------------------------------------------------------
// transposes and setup
// ---------------------------------------------------------------------------
// Copies the value of every node of a field from family `fs` (src) to the
// other (dst).  Reads run along the source diagonals (contiguous), writes
// scatter.
template <int MB>
__device__ inline void d_transpose(const DGeom& g, const float* src, float* dst, int fs,
                                   int lane) {
  for (int d = 0; d < g.nd; ++d) {
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      const int j = lane + 32 * m;
      const int i = fs == 0 ? d - j : d + j - (g.ny - 1);
      if (j < g.ny && i >= 0 && i < g.nx)
        dst[dix(g, 1 - fs, i, j)] = src[(d + 1) * g.pitch + j];
    }
  }
  __syncwarp();
}

// T0 and its gradient of every node into both families; tau[0] initialised
// (1 in the frozen box).
template <int MB>
__device__ inline void d_t0(const PeriodDev& P, const DGeom& g, double x0, double y0,
                            const WSolve& w, const DSlot& V, int lane) {
  const T0Src src = t0_source(w, x0, y0);
  for (int i = lane; i < g.nx; i += 32) {
    const float hx = (float)((P.xs[i] - x0) * 0.5);
    V.col[i] = sinf(hx);
    V.col[g.nx + i] = cosf(hx);
  }
  __syncwarp();
  T0Row row[MB];
#pragma unroll
  for (int m = 0; m < MB; ++m) {
    const int j = lane + 32 * m;
    if (j < g.ny) row[m] = t0_row(P, src, j);
  }
  for (int d = 0; d < g.nd; ++d) {
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      const int j = lane + 32 * m, i = d - j;
      if (j < g.ny && i >= 0 && i < g.nx) {
        const float4 s = t0_cell(P, src, row[m], i, j, V.col[i], V.col[g.nx + i]);
        const int a = (d + 1) * g.pitch + j, b = dix(g, 1, i, j);
        V.t0[0][a] = s.x;
        V.t0[1][b] = s.x;
        V.gxy[0][a] = make_float2(s.y, s.z);
        V.gxy[1][b] = make_float2(s.y, s.z);
        V.tau[0][a] = w.box.has(i, j) ? 1.0f : 10.0f;
      }
    }
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// forward sweeps
// ---------------------------------------------------------------------------
// Layout row holding step `tau` (0 .. nd) of a forward sweep.
__device__ __forceinline__ int df_row(const DGeom& g, int tau, int xdir) {
  return xdir > 0 ? tau + 1 : g.nd - tau;
}
// Element of logical row v in a diagonal; lanes past the grid's last row
// (the band count follows the tallest grid of the evaluation) read row ny-1
// and discard it.
__device__ __forceinline__ int df_col(const DGeom& g, int v, int ydir) {
  return v >= g.ny ? g.ny - 1 : (ydir > 0 ? v : g.ny - 1 - v);
}

// Arrays of one forward sweep, in the sweep's family.
struct DFwdArrays {
  float* tau;
  const float* t0;
  const float2* gxy;
  const float4* qa;
  const float2* qd;
  float* old;  // family 0
};

// The value and T0 of a cell, what the lanes exchange.
struct DLight {
  bool on, frz;
  float own, t0;
};

// lane 0: fill number ring.next with the rows of step `tau`.
template <int NS, int PM>
__device__ inline void df_fill(const Ring<NS>& ring, const DGeom& g, const DFwdArrays& R, int tau,
                               int xdir, bool last) {
  const size_t off = (size_t)df_row(g, tau, xdir) * g.pitch;
  const unsigned P = (unsigned)g.pitch;
  const uint32_t s = smem_u32(ring.stage(ring.next));
  const uint32_t b = ring.bar(ring.next);
  mbar_expect_tx(b, P * (last ? 44u : 40u));
  bulk_g2s(s, R.tau + off, 4 * P, b);
  bulk_g2s(s + kStOffT0 * PM, R.t0 + off, 4 * P, b);
  bulk_g2s(s + kStOffGxy * PM, R.gxy + off, 8 * P, b);
  bulk_g2s(s + kStOffQa * PM, R.qa + off, 16 * P, b);
  bulk_g2s(s + kStOffQd * PM, R.qd + off, 8 * P, b);
  if (last) bulk_g2s(s + kStOffOld * PM, R.old + off, 4 * P, b);
}

template <int PM>
__device__ __forceinline__ DLight df_light(const char* st, const DGeom& g, int t, int v, int xdir,
                                           int ydir, const Box& box) {
  DLight o;
  const int u = t - v;
  o.on = v < g.ny && u >= 0 && u < g.nx;
  o.frz = box.has(xdir > 0 ? u : g.nx - 1 - u, ydir > 0 ? v : g.ny - 1 - v);
  const int jj = df_col(g, v, ydir);
  o.own = reinterpret_cast<const float*>(st)[jj];
  o.t0 = reinterpret_cast<const float*>(st + kStOffT0 * PM)[jj];
  return o;
}

// Returns false when a stage did not arrive (bounded wait).
template <int MB, int NS>
__device__ inline bool d_fwd_sweeps(const PeriodDev& P, const DGeom& g, const DSlot& V,
                                    const WSolve& w, Ring<NS>& ring, int lane, int* status_out,
                                    int* iters_out) {
  constexpr int PM = 32 * MB;
  const int nx = g.nx, ny = g.ny;
  const float idx = (float)(1.0 / P.dx), idy = (float)(1.0 / P.dy);
  const int nsteps = g.nd;  // steps 0 .. nd-1, operands of steps 0 .. nd
  int iter, status = ST_NOT_CONVERGED;
  for (iter = 1; iter <= MAXITER_UW; ++iter) {
    float l1 = 0.f, lmax = 0.f;
    for (int s = 0; s < 4; ++s) {
      int xdir, ydir;
      sweep_dirs(s, xdir, ydir);
      const int fam = xdir == ydir ? 0 : 1;
      if (s == 1) d_transpose<MB>(g, V.tau[0], V.tau[1], 0, lane);
      if (s == 3) d_transpose<MB>(g, V.tau[1], V.tau[0], 1, lane);
      const bool last = s == 3;
      DFwdArrays R;
      R.tau = fam ? V.tau[1] : V.tau[0];
      R.t0 = fam ? V.t0[1] : V.t0[0];
      R.gxy = fam ? V.gxy[1] : V.gxy[0];
      R.qa = fam ? P.qa[1] : P.qa[0];
      R.qd = fam ? P.qd[1] : P.qd[0];
      R.old = V.old;
      // this warp's earlier global writes become visible to the bulk copies
      fence_async_global();
      __syncwarp();
      const unsigned long long base = ring.next;
      for (int k = 0; k < NS && k <= nsteps; ++k) {
        if (lane == 0) df_fill<NS, PM>(ring, g, R, k, xdir, last);
        ++ring.next;
      }
      if (!ring.wait(base)) {
        ring.drain(base);
        return false;
      }
      float res[MB], t0prev[MB];
      DLight cur[MB];
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        res[m] = 0.f;
        t0prev[m] = 0.f;
        cur[m] = df_light<PM>(ring.stage(base), g, 0, lane + 32 * m, xdir, ydir, w.box);
      }
      for (int t = 0; t < nsteps; ++t) {
        const unsigned long long n1 = base + t + 1;
        if (!ring.wait(n1)) {
          ring.drain(n1);
          return false;
        }
        const char* s0 = ring.stage(base + t);
        const char* s1 = ring.stage(n1);
        if (lane == 0 && t + NS + 4 <= nsteps) {
          // further ahead: the rows into L2
          const size_t off = (size_t)df_row(g, t + NS + 4, xdir) * g.pitch;
          const unsigned p4 = 4u * g.pitch;
          l2_prefetch(R.tau + off, p4);
          l2_prefetch(R.t0 + off, p4);
          l2_prefetch(R.gxy + off, 2 * p4);
          l2_prefetch(R.qa + off, 4 * p4);
          l2_prefetch(R.qd + off, 2 * p4);
        }
        DLight nxt[MB];
        float south[MB], t0s[MB], north[MB], t0n[MB], nown[MB], nt0[MB];
#pragma unroll
        for (int m = 0; m < MB; ++m) {
          nxt[m] = df_light<PM>(s1, g, t + 1, lane + 32 * m, xdir, ydir, w.box);
          nown[m] = nxt[m].own;
          nt0[m] = nxt[m].t0;
        }
        w_from_below<MB>(res, south, lane);
        w_from_below<MB>(t0prev, t0s, lane);
        w_from_above<MB>(nown, north, lane);
        w_from_above<MB>(nt0, t0n, lane);
        const int row = df_row(g, t, xdir);
#pragma unroll
        for (int m = 0; m < MB; ++m) {
          const int v = lane + 32 * m, u = t - v;
          const int jj = df_col(g, v, ydir);
          WFwd o;
          o.own = cur[m].own;
          o.t0 = cur[m].t0;
          const float2 gv = reinterpret_cast<const float2*>(s0 + kStOffGxy * PM)[jj];
          o.gx = gv.x;
          o.gy = gv.y;
          o.pa = reinterpret_cast<const float4*>(s0 + kStOffQa * PM)[jj];
          const float2 dv = reinterpret_cast<const float2*>(s0 + kStOffQd * PM)[jj];
          o.dsx = dv.x;
          o.dsy = dv.y;
          float nv = wf_visit(o, res[m], nown[m], south[m], north[m], t0prev[m], nt0[m], t0s[m],
                              t0n[m], u > 0, v > 0, u < nx - 1, v < ny - 1, xdir, ydir, idx, idy);
          nv = cur[m].frz ? cur[m].own : nv;
          if (cur[m].on) {
            const int a = row * g.pitch + jj;
            R.tau[a] = nv;
            if (s == 0) R.old[a] = cur[m].own;
            if (last && !cur[m].frz) {
              const float old = reinterpret_cast<const float*>(s0 + kStOffOld * PM)[jj];
              const float dd = fabsf(nv - old) * cur[m].t0;
              l1 += dd;
              lmax = fmaxf(lmax, dd);
            }
            res[m] = nv;
            t0prev[m] = cur[m].t0;
          }
          cur[m] = nxt[m];
        }
        __syncwarp();
        // the stage of step t is free: fill it with step t + NS
        if (t + NS <= nsteps) {
          // every lane has consumed its reads of the stage (their values fed
          // this step's updates) before __syncwarp, so the copy may overwrite it
          if (lane == 0) df_fill<NS, PM>(ring, g, R, t + NS, xdir, last);
          ++ring.next;
        }
      }
    }
    // FP64 decision over the lanes' partial sums (src/eikon_solver_2d.f90:1091-1115)
    double sl1 = (double)l1, smax = (double)lmax;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sl1 += __shfl_xor_sync(FULL, sl1, o);
      smax = fmax(smax, __shfl_xor_sync(FULL, smax, o));
    }
    sl1 = sl1 / (double)nx / (double)ny;
    if (fabs(sl1) < TOL_UW && smax < TOL_UW) {
      status = ST_OK;
      break;
    }
  }
  *status_out = status;
  *iters_out = iter > MAXITER_UW ? MAXITER_UW : iter;
  return true;
}

// ---------------------------------------------------------------------------
// adjoint
// ---------------------------------------------------------------------------
// Weights and 1/d of every node along the family-0 diagonals: the 3x3
// stencil of a node lies on diagonals d-2 .. d+2, read contiguously across
// the lanes.
template <int MB>
__device__ inline void d_adj_setup(const PeriodDev& P, const DGeom& g, const DSlot& V, int lane) {
  const int nx = g.nx, ny = g.ny, pitch = g.pitch;
  const float idx = (float)(1.0 / P.dx), idy = (float)(1.0 / P.dy);
  const float* tau = V.tau[0];
  const float* T0 = V.t0[0];
  const float4* PA = P.qa[0];
  for (int d = 0; d < g.nd; ++d) {
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      const int j = lane + 32 * m, i = d - j;
      if (!(j < ny && i >= 0 && i < nx)) continue;
      const int k = (d + 1) * pitch + j;
      const int kb = dix(g, 1, i, j);
      if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1) {
        V.W[0][k] = make_float4(0.f, 0.f, 0.f, 0.f);
        V.W[1][kb] = make_float4(0.f, 0.f, 0.f, 0.f);
        V.id[k] = 0.f;
        continue;
      }
      // node (i + di, j + dj) of family 0
      auto at = [&](int di, int dj) { return k + (di + dj) * pitch + dj; };
      auto T = [&](int q) { return __fmul_rn(tau[q], T0[q]); };
      const int w = at(-1, 0), e = at(1, 0), s = at(0, -1), n = at(0, 1);
      const float4 pk = PA[k], pw = PA[w], pe = PA[e], ps = PA[s], pn = PA[n];
      const float Tk = T(k), Tw = T(w), Te = T(e), Ts = T(s), Tn = T(n);
      const float Twn = T(at(-1, 1)), Tws = T(at(-1, -1)), Ten = T(at(1, 1)), Tes = T(at(1, -1));
      float4 W;
      const float id = adj_weights(Tk, Tw, Te, Ts, Tn, Twn, Tws, Ten, Tes, pk, pw, pe, ps, pn, idx,
                                   idy, &W);
      V.W[0][k] = W;
      V.W[1][kb] = W;
      V.id[k] = id;
    }
  }
  __syncwarp();
}

// Layout row holding step `tau` (0 .. nu+nv-1) of an adjoint sweep, and the
// element of interior logical row v (lanes past the last interior row read
// row ny-2 and discard it).
__device__ __forceinline__ int da_row(const DGeom& g, int tau, int xdir) {
  return xdir > 0 ? tau + 3 : g.nd - 2 - tau;
}
__device__ __forceinline__ int da_col(const DGeom& g, int v, int nv, int ydir) {
  return v >= nv ? g.ny - 2 : (ydir > 0 ? 1 + v : g.ny - 2 - v);
}

// Arrays of one adjoint sweep, in the sweep's family.
struct DAdjArrays {
  float* tau;
  const float4* W;
  const float* src;
  float* old;  // family 0
};

template <int NS, int PM>
__device__ inline void da_fill(const Ring<NS>& ring, const DGeom& g, const DAdjArrays& R, int tau,
                               int xdir, bool last) {
  const size_t off = (size_t)da_row(g, tau, xdir) * g.pitch;
  const unsigned P = (unsigned)g.pitch;
  const uint32_t s = smem_u32(ring.stage(ring.next));
  const uint32_t b = ring.bar(ring.next);
  mbar_expect_tx(b, P * (last ? 28u : 24u));
  bulk_g2s(s, R.tau + off, 4 * P, b);
  bulk_g2s(s + kStOffT0 * PM, R.src + off, 4 * P, b);
  bulk_g2s(s + kStOffQa * PM, R.W + off, 16 * P, b);
  if (last) bulk_g2s(s + kStOffOld * PM, R.old + off, 4 * P, b);
}

// Sweeps one adjoint field (sources src0 / src1 per family) to convergence:
// the reference's absolute rule (:1429) or no change beyond the FP32
// resolution of the field.  Neighbours outside the interior are the
// boundary's zeros.  Returns false when a stage did not arrive.
template <int MB, int NS>
__device__ inline bool d_adj_sweeps(const DGeom& g, const DSlot& V, const float* src0,
                                    const float* src1, Ring<NS>& ring, int lane, int* status_out,
                                    int* iters_out) {
  constexpr int PM = 32 * MB;
  const int nx = g.nx, ny = g.ny;
  const int nu = nx - 2, nv = ny - 2;
  const int nsteps = nu + nv - 1;
  for (int d = 0; d < g.nd; ++d)
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      const int j = lane + 32 * m, i = d - j;
      if (j < ny && i >= 0 && i < nx) {
        const bool in = i > 0 && i < nx - 1 && j > 0 && j < ny - 1;
        V.tau[0][(d + 1) * g.pitch + j] = in ? 100.f : 0.f;
      }
    }
  __syncwarp();
  int iter, status = ST_NOT_CONVERGED;
  for (iter = 1; iter <= MAXITER_JSE; ++iter) {
    float l1 = 0.f, lmax = 0.f, vmax = 0.f;
    for (int s = 0; s < 4; ++s) {
      int xdir, ydir;
      sweep_dirs(s, xdir, ydir);
      const int fam = xdir == ydir ? 0 : 1;
      if (s == 1) d_transpose<MB>(g, V.tau[0], V.tau[1], 0, lane);
      if (s == 3) d_transpose<MB>(g, V.tau[1], V.tau[0], 1, lane);
      const bool last = s == 3;
      DAdjArrays R;
      R.tau = fam ? V.tau[1] : V.tau[0];
      R.W = fam ? V.W[1] : V.W[0];
      R.src = fam ? src1 : src0;
      R.old = V.old;
      fence_async_global();
      __syncwarp();
      const unsigned long long base = ring.next;
      for (int k = 0; k < NS && k <= nsteps; ++k) {
        if (lane == 0) da_fill<NS, PM>(ring, g, R, k, xdir, last);
        ++ring.next;
      }
      if (!ring.wait(base)) {
        ring.drain(base);
        return false;
      }
      float res[MB], cown[MB];
#pragma unroll
      for (int m = 0; m < MB; ++m) {
        const int v = lane + 32 * m;
        res[m] = 0.f;
        cown[m] = reinterpret_cast<const float*>(ring.stage(base))[da_col(g, v, nv, ydir)];
      }
      for (int t = 0; t < nsteps; ++t) {
        const unsigned long long n1 = base + t + 1;
        if (!ring.wait(n1)) {
          ring.drain(n1);
          return false;
        }
        const char* s0 = ring.stage(base + t);
        const char* s1 = ring.stage(n1);
        if (lane == 0 && t + NS + 4 <= nsteps) {
          const size_t off = (size_t)da_row(g, t + NS + 4, xdir) * g.pitch;
          const unsigned p4 = 4u * g.pitch;
          l2_prefetch(R.tau + off, p4);
          l2_prefetch(R.src + off, p4);
          l2_prefetch(R.W + off, 4 * p4);
        }
        float south[MB], north[MB], nown[MB];
#pragma unroll
        for (int m = 0; m < MB; ++m) {
          const int v = lane + 32 * m;
          nown[m] = reinterpret_cast<const float*>(s1)[da_col(g, v, nv, ydir)];
        }
        w_from_below<MB>(res, south, lane);
        w_from_above<MB>(nown, north, lane);
        const int row = da_row(g, t, xdir);
#pragma unroll
        for (int m = 0; m < MB; ++m) {
          const int v = lane + 32 * m, u = t - v;
          const int jj = da_col(g, v, nv, ydir);
          const bool on = v < nv && u >= 0 && u < nu;
          const float west = u > 0 ? res[m] : 0.f;
          const float east = u < nu - 1 ? nown[m] : 0.f;
          const float sth = v > 0 ? south[m] : 0.f;
          const float nth = v < nv - 1 ? north[m] : 0.f;
          const float tw = xdir > 0 ? west : east, te = xdir > 0 ? east : west;
          const float ts = ydir > 0 ? sth : nth, tn = ydir > 0 ? nth : sth;
          const float4 W = reinterpret_cast<const float4*>(s0 + kStOffQa * PM)[jj];
          const float sv = reinterpret_cast<const float*>(s0 + kStOffT0 * PM)[jj];
          const float val = adj_update(sv, W, tw, te, ts, tn);
          if (on) {
            const int a = row * g.pitch + jj;
            R.tau[a] = val;
            if (s == 0) R.old[a] = cown[m];
            if (last) {
              const float old = reinterpret_cast<const float*>(s0 + kStOffOld * PM)[jj];
              const float dd = fabsf(val - old);
              l1 += dd;
              lmax = fmaxf(lmax, dd);
              vmax = fmaxf(vmax, fabsf(val));
            }
            res[m] = val;
          }
          cown[m] = nown[m];
        }
        __syncwarp();
        if (t + NS <= nsteps) {
          if (lane == 0) da_fill<NS, PM>(ring, g, R, t + NS, xdir, last);
          ++ring.next;
        }
      }
    }
    double sl1 = (double)l1, smax = (double)lmax, svmax = (double)vmax;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sl1 += __shfl_xor_sync(FULL, sl1, o);
      smax = fmax(smax, __shfl_xor_sync(FULL, smax, o));
      svmax = fmax(svmax, __shfl_xor_sync(FULL, svmax, o));
    }
    sl1 = sl1 / (double)(nx * ny);
    if ((fabs(sl1) < TOL_JSE && smax < TOL_JSE) || smax <= svmax * 0x1p-21) {
      status = ST_OK;
      break;
    }
  }
  *status_out = status;
  *iters_out = iter > MAXITER_JSE ? MAXITER_JSE : iter;
  return true;
}

// T = tau*T0 at node (i, j) (FP64 product of the FP32 factors)
__device__ __forceinline__ double d_T(const DGeom& g, const DSlot& V, int i, int j) {
  const int k = dix(g, 0, i, j);
  return (double)V.tau[0][k] * (double)V.t0[0][k];
}

// interp2_0_dp on the caller's increasing degree grid (src/shared/utils.f90:917-942)
__device__ inline bool d_interp(const PeriodDev& P, const DGeom& g, const DSlot& V, double xq,
                                double yq, double* out) {
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
  r = r + d_T(g, V, x1, y1) * (n1 / vn);
  r = r + d_T(g, V, x2, y1) * (n2 / vn);
  r = r + d_T(g, V, x1, y2) * (n3 / vn);
  r = r + d_T(g, V, x2, y2) * (n4 / vn);
  *out = r;
  return true;
}

// ---------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------
// Bytes of the dynamic shared memory of one block (the stage ring).
template <int MB, int NS>
constexpr int d_smem_bytes() {
  return NS * kStageBytesPerElem * 32 * MB;
}

// One warp per block; MINW resident warps per SM is the launch bound (8: 255
// registers a thread, 12: 168), NS the stages of the ring.
template <int MB, int NS, int MINW>
__global__ void __launch_bounds__(32, MINW) k_batch_fp32d(BatchArgs A) {
  extern __shared__ __align__(128) char dsm[];
  __shared__ __align__(8) unsigned long long bars[NS];
  const int lane = threadIdx.x & 31;
  double* base = A.ws + (long long)blockIdx.x * A.ws_doubles;
  float* kf = reinterpret_cast<float*>(A.kcontrib);
  float* kdf = reinterpret_cast<float*>(A.kcontrib_den);
  Ring<NS> ring;
  ring.base = dsm;
  ring.bar0 = smem_u32(&bars[0]);
  ring.stage_bytes = kStageBytesPerElem * 32 * MB;
  ring.next = 0;
  ring.wait_cycles = A.phase_cycles ? A.phase_cycles + PH_WAIT : nullptr;
  if (lane == 0) {
    for (int k = 0; k < NS; ++k) mbar_init(ring.bar0 + 8u * k, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  for (;;) {
    int q = 0;
    if (lane == 0) q = atomicAdd(A.queue, 1);
    q = __shfl_sync(FULL, q, 0);
    if (q >= A.nsolve) break;
    const int s = A.order[q];
    const PeriodDev P = A.periods[A.pidx[s]];
    const int nx = P.nx, ny = P.ny;
    const size_t N = (size_t)nx * ny;
    const DGeom g{nx, ny, diag_pitch(ny), nx + ny - 1};
    const long long D = diag_cells(nx, ny);
    const int r0 = A.rec_off[s], nr = A.nrec[s];
    const DSlot V = dcarve(base, D);
    const double xd0 = A.srcx[s], yd0 = A.srcy[s];
    const double x0 = xd0 / 180.0 * PI_S, y0 = yd0 / 180.0 * PI_S;
    unsigned long long* const pc = A.phase_cycles;
    long long c0 = pc ? clock64() : 0;
    // adds the cycles since the previous mark to phase `ph` (lane 0, when on)
    auto mark = [&](int ph) {
      if (pc) {
        const long long c1 = clock64();
        if (lane == 0) atomicAdd(pc + ph, (unsigned long long)(c1 - c0));
        c0 = c1;
      }
    };
    // a stage that did not arrive: report, and stop this warp
    auto timed_out = [&]() {
      if (lane == 0) {
        A.status[s] = ST_TIMEOUT;
        A.fwd_iters[s] = 0;
        A.adj_iters[s] = 0;
      }
      __syncwarp();
    };
    const WSolve w = w_locate(P, x0, y0, xd0, yd0, lane);
    if (w.status != ST_OK) {
      for (int r = lane; r < nr; r += 32) {
        A.tekio[r0 + r] = 0.0;
        A.wgt_eff[r0 + r] = 0.0;
        A.tt_fwd[A.path[r0 + r]] = 0.0;
      }
      if (A.mode >= 2)
        for (size_t k = lane; k < N; k += 32) {
          kf[A.kslot[s] + k] = 0.f;
          if (A.mode == 3) kdf[A.kslot[s] + k] = 0.f;
        }
      if (lane == 0) {
        A.chi[s] = 0.0;
        A.status[s] = w.status;
        A.fwd_iters[s] = 0;
        A.adj_iters[s] = 0;
        if (A.fwd_updates) A.fwd_updates[s] = 0;
      }
      __syncwarp();
      continue;
    }
    d_t0<MB>(P, g, x0, y0, w, V, lane);
    mark(PH_SETUP);
    int fst = ST_OK, fit = 0;
    if (!d_fwd_sweeps<MB, NS>(P, g, V, w, ring, lane, &fst, &fit)) {
      timed_out();
      return;
    }
    mark(PH_FWD);
    if (A.fwd_updates && lane == 0) {
      const double frozen = (double)(w.box.i1 - w.box.i0 + 1) * (w.box.j1 - w.box.j0 + 1);
      A.fwd_updates[s] = (double)fit * 4.0 * ((double)N - frozen);
    }
    // receiver times, misfit, outlier weights (src/measadj.f90:71-72, 82-84)
    int bad = 0;
    for (int r = lane; r < nr; r += 32) {
      double v = 0.0;
      if (!d_interp(P, g, V, A.recx[r0 + r], A.recy[r0 + r], &v)) bad = 1;
      A.tekio[r0 + r] = v;
      A.tt_fwd[A.path[r0 + r]] = v;
    }
    bad = __any_sync(FULL, bad);
    __syncwarp();
    if (lane == 0) {
      double ssum = 0;
      for (int r = 0; r < nr; ++r) {
        const double dd = A.tekio[r0 + r] - A.tt[r0 + r];
        ssum = ssum + A.weight[r0 + r] * (dd * dd);
      }
      A.chi[s] = 0.5 * ssum;
      for (int r = 0; r < nr; ++r) {
        double wt = A.weight[r0 + r];
        if (fabs(A.tekio[r0 + r] - A.tt[r0 + r]) / A.tt[r0 + r] > 0.5) wt = 0.;
        A.wgt_eff[r0 + r] = wt;
      }
    }
    __syncwarp();
    mark(PH_RECV);
    int st = fst;
    if (bad && st == ST_OK) st = ST_BAD_ARG;
    int aiters = 0;
    if (A.mode >= 2) {
      const int nf = A.mode == 3 ? 2 : 1;
      d_adj_setup<MB>(P, g, V, lane);
      for (int f = 0; f < nf; ++f) {
        float* sf = f ? V.src[1][0] : V.src[0][0];
        for (long long k = lane; k < D; k += 32) sf[k] = 0.f;
      }
      __syncwarp();
      // adjoint sources weight*(tekio-tt) (src/measadj.f90:88) and -weight
      // (:102), bilinear splat over the cell area (:1328-1336), scaled by 1/d
      st = adj_sources_warp(A, P, r0, nr, nf, V.src[0][0], V.src[nf - 1][0], V.id,
                            [&g](int i, int j) { return dix(g, 0, i, j); }, lane, st);
      st = __shfl_sync(FULL, st, 0);
      __syncwarp();
      for (int f = 0; f < nf; ++f)
        d_transpose<MB>(g, f ? V.src[1][0] : V.src[0][0], f ? V.src[1][1] : V.src[0][1], 0, lane);
      mark(PH_ADJ_SETUP);
      int its[2] = {0, 0};
      for (int f = 0; f < nf; ++f) {
        int ast = ST_OK;
        if (!d_adj_sweeps<MB, NS>(g, V, f ? V.src[1][0] : V.src[0][0],
                                  f ? V.src[1][1] : V.src[0][1], ring, lane, &ast, &its[f])) {
          timed_out();
          return;
        }
        mark(PH_ADJ);
        if (ast != ST_OK && st == ST_OK) st = ast;
        // mask (:1449-1467) and the slot adj/svel**k (:314-315), FP32 here,
        // summed per period in FP64
        float* out = (f == 0 ? kf : kdf) + A.kslot[s];
        for (int j = 0; j < ny; ++j)
          for (int i = lane; i < nx; i += 32) {
            const size_t k = i + (size_t)nx * j;
            const float4 pb = P.p4b[k];
            const float isv = A.mode == 3 ? pb.w : pb.z;
            out[k] = w.mbox.has(i, j) ? 0.f : V.tau[0][dix(g, 0, i, j)] * isv;
          }
        __syncwarp();
        mark(PH_SLOT);
      }
      aiters = its[0] > its[1] ? its[0] : its[1];
      if (A.adj_updates && lane == 0)
        A.adj_updates[s] = (double)(its[0] + its[1]) * 4.0 * (nx - 2) * (ny - 2);
    }
    if (lane == 0) {
      A.status[s] = st;
      A.fwd_iters[s] = fit;
      A.adj_iters[s] = aiters;
    }
    __syncwarp();
  }
}

// Variants: (stages, resident warps per SM)
//   0: 3 stages, 12 warps      1: 3 stages, 8 warps      2: 4 stages, 8 warps
constexpr int kFp32dVariants = 3;
int fp32d_variant_count() { return kFp32dVariants; }

template <int MB, int NS, int MINW>
static void launch_d(const BatchArgs& a, int grid, cudaStream_t st) {
  k_batch_fp32d<MB, NS, MINW><<<grid, 32, d_smem_bytes<MB, NS>(), st>>>(a);
}

template <int MB, int NS, int MINW>
static int occupancy_d() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_fp32d<MB, NS, MINW>, 32,
                                                d_smem_bytes<MB, NS>());
  return n;
}

template <int MB>
static void launch_dmb(const BatchArgs& a, int grid, int variant, cudaStream_t st) {
  switch (variant) {
    case 0: launch_d<MB, 3, 12>(a, grid, st); break;
    case 1: launch_d<MB, 3, 8>(a, grid, st); break;
    default: launch_d<MB, 4, 8>(a, grid, st); break;
  }
}

template <int MB>
static int occupancy_dmb(int variant) {
  switch (variant) {
    case 0: return occupancy_d<MB, 3, 12>();
    case 1: return occupancy_d<MB, 3, 8>();
    default: return occupancy_d<MB, 4, 8>();
  }
}

void launch_batch_fp32d(const BatchArgs& a, int grid, int bands, int variant, cudaStream_t st) {
  switch (bands) {
    case 1: launch_dmb<1>(a, grid, variant, st); break;
    case 2: launch_dmb<2>(a, grid, variant, st); break;
    case 3: launch_dmb<3>(a, grid, variant, st); break;
    default: launch_dmb<4>(a, grid, variant, st); break;
  }
}

int batch_fp32d_max_blocks_per_sm(int bands, int variant) {
  switch (bands) {
    case 1: return occupancy_dmb<1>(variant);
    case 2: return occupancy_dmb<2>(variant);
    case 3: return occupancy_dmb<3>(variant);
    default: return occupancy_dmb<4>(variant);
  }
}

}  // namespace sgb
