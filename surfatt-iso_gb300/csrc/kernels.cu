// kernels.cu -- FP64 kernels: per-period precompute, the fused batched
// (period, source) solve, ordered kernel / misfit reductions, and the
// single-solve kernels behind the drop-in symbols.
#include <cstdio>

#include <algorithm>

#include <cooperative_groups.h>

#include "kernels.cuh"
#include "solver_fp64.cuh"
#include "batch_tail.cuh"

namespace sgb {

// ---------------------------------------------------------------------------
// Per-period precompute (one block row per period field).
// lon/lat: xx = xx_deg/180.0*pi (:801-804); a = spha/(R^2 cos^2 y),
// b = sphb/R^2, c = sphc/(R^2 cos y) (:817-821).  The one-sided `dis` terms
// (:1014, :1055) are loop invariant and evaluated here exactly as written.
// ---------------------------------------------------------------------------
__device__ inline void prep_cells(const PrepIn& in, const PrepOut& out, size_t tid, size_t nthr) {
  const int nx = in.nx, ny = in.ny;
  const size_t N = (size_t)nx * ny;
  if (out.xs)  // axis outputs are optional (already prepared for this grid)
    for (size_t i = tid; i < (size_t)nx; i += nthr)
      out.xs[i] = in.lonlat ? in.xdeg[i] / 180.0 * PI_S : in.xdeg[i];
  if (out.ys)
    for (size_t j = tid; j < (size_t)ny; j += nthr) {
      const double y = in.lonlat ? in.ydeg[j] / 180.0 * PI_S : in.ydeg[j];
      out.ys[j] = y;
      if (in.lonlat) {
        out.cosy[j] = cos(y);
        out.siny[j] = sin(y);
      }
    }
  for (size_t k = tid; k < N; k += nthr) {
    const int j = (int)(k / nx);
    double A = in.A[k], B = in.B[k], C = in.C[k], f;
    if (in.from_model) {
      C = -C;
      f = 1. / in.V[k];
    } else {
      f = in.V[k];
    }
    double a = A, b = B, c = C;
    if (in.lonlat) {
      const double y = in.ydeg[j] / 180.0 * PI_S;
      const double cy = cos(y);
      a = A / (R_EARTH * R_EARTH * (cy * cy));
      b = B / (R_EARTH * R_EARTH);
      c = C / (R_EARTH * R_EARTH * cy);
    }
    out.a[k] = a;
    out.b[k] = b;
    out.c[k] = c;
    out.fun[k] = f;
    out.f2[k] = f * f;
    out.disx[k] = sqrt(f * f * (b / (a * b - c * c)));
    out.disy[k] = sqrt(f * f * (a / (a * b - c * c)));
    if (out.f32) {
      out.f32[k] = (float)a;
      out.f32[N + k] = (float)b;
      out.f32[2 * N + k] = (float)c;
      out.f32[3 * N + k] = (float)(f * f);
      out.f32[4 * N + k] = (float)out.disx[k];
      out.f32[5 * N + k] = (float)out.disy[k];
    }
    if (out.isv && in.from_model) {
      const double v = in.V[k];
      out.isv[k] = 1.0 / (v * v);
      out.isv[N + k] = 1.0 / (v * v * v);
    }
    if (out.p4a) out.p4a[2 * k] = make_float4((float)a, (float)b, (float)c, (float)(f * f));
    if (out.p4b) {
      float i2 = 0.f, i3 = 0.f;
      if (in.from_model) {
        const double v = in.V[k];
        i2 = (float)(1.0 / (v * v));
        i3 = (float)(1.0 / (v * v * v));
      }
      out.p4b[2 * k] = make_float4((float)out.disx[k], (float)out.disy[k], i2, i3);
    }
  }
}

__global__ void k_prep(PrepIn in, PrepOut out) {
  prep_cells(in, out, blockIdx.x * (size_t)blockDim.x + threadIdx.x,
             (size_t)gridDim.x * blockDim.x);
}

// Up to kPrepBatch periods in one launch (block row p: period p), so that a
// load or a velocity update of many small periods is one launch, not one
// per period.  The table travels as the kernel's parameter.
constexpr int kPrepBatch = 32;
struct PrepBatch {
  int n;
  PrepIn in[kPrepBatch];
  PrepOut out[kPrepBatch];
};

__global__ void k_prep_batch(const __grid_constant__ PrepBatch b) {
  const int p = blockIdx.y;
  if (p >= b.n) return;
  prep_cells(b.in[p], b.out[p], blockIdx.x * (size_t)blockDim.x + threadIdx.x,
             (size_t)gridDim.x * blockDim.x);
}

static int prep_grid(size_t N) {
  int grid = (int)((N + 255) / 256);
  if (grid < 1) grid = 1;
  if (grid > 4096) grid = 4096;
  return grid;
}

void launch_prep(const PrepIn& in, const PrepOut& out, cudaStream_t st) {
  k_prep<<<prep_grid((size_t)in.nx * in.ny), 256, 0, st>>>(in, out);
}

void launch_prep_batch(const PrepIn* in, const PrepOut* out, int np, cudaStream_t st) {
  for (int p0 = 0; p0 < np; p0 += kPrepBatch) {
    PrepBatch b;
    b.n = np - p0 < kPrepBatch ? np - p0 : kPrepBatch;
    size_t nmax = 0;
    for (int i = 0; i < b.n; ++i) {
      b.in[i] = in[p0 + i];
      b.out[i] = out[p0 + i];
      nmax = std::max(nmax, (size_t)in[p0 + i].nx * in[p0 + i].ny);
    }
    k_prep_batch<<<dim3(prep_grid(nmax), b.n), 256, 0, st>>>(b);
  }
}

// ---------------------------------------------------------------------------
// Fused batched solve (FP64).  Persistent blocks pull solves from a device
// work queue; each runs forward -> interp2 -> misfit -> adjoint(s) -> mask
// -> kernel contribution for one (period, source).
// ---------------------------------------------------------------------------
// tau, tau_old, T0, T + max(forward constants, adjoint constants + 6 fields)
__host__ __device__ constexpr long long fp64_slot_doubles(long long N) {
  return (4 + ((long long)KC_COUNT > (long long)KA_COUNT + 6 ? (long long)KC_COUNT
                                                              : (long long)KA_COUNT + 6)) * N;
}

long long batch_fp64_ws_doubles(long long N) { return fp64_slot_doubles(N); }

struct SolveLayout {
  FwdWs fw;
  AdjWs aw;
  double* T;
};

__device__ inline SolveLayout carve(double* base, size_t N) {
  SolveLayout L;
  L.fw.tau = base;
  L.fw.tau_old = base + N;
  L.fw.T0 = base + 2 * N;
  L.T = base + 3 * N;
  L.fw.K = base + 4 * N;
  L.aw.T = L.T;
  L.aw.K = base + 4 * N;  // aliases the forward constants (dead by then)
  double* f = base + 4 * N + KA_COUNT * N;
  L.aw.delta[0] = f;
  L.aw.delta[1] = f + N;
  L.aw.Ta[0] = f + 2 * N;
  L.aw.Ta[1] = f + 3 * N;
  L.aw.old[0] = f + 4 * N;
  L.aw.old[1] = f + 5 * N;
  return L;
}

// With A.items == kFp64Items a solve is cut into work items as in the FP32
// row kernel: the queue hands out every solve's item 0, then every item 1,
// ..., so the last round of a batch is one short item rather than whole
// solves (1280 solves on 608 resident blocks are 2.1 rounds of whole
// solves: a third of the last round's SMs would idle).  Items 0 ..
// kFp64Items - 2 run kFp64SplitIter forward iterations; the last runs the
// sweeps to convergence and the solve's tail (receivers, misfit, adjoints,
// mask, kernel slot).  tau, T0 and the T0 gradient persist between items
// in the solve's own arrays (A.ws_solve: four planes of solve_cells
// doubles, the solve at its kernel-slot offset); every later item rebuilds
// only the hoisted constants in its block's scratch, to the same bits, so
// the results equal the whole-solve kernel's.  An item waits,
// bounded, for its solve's previous item (taken earlier by a resident
// block); running out reports SURFATT_TIMEOUT for the solve.
__global__ void __launch_bounds__(128) k_batch_fp64(BatchArgs A) {
  __shared__ SolveShared sh;
  __shared__ int next, prev_done, prev_fit, prev_fst;
  double* base = A.ws + (size_t)blockIdx.x * (size_t)A.ws_doubles;
  const bool cut = A.items > 1;
  const int nitem = cut ? A.items : 1;
  for (;;) {
    if (threadIdx.x == 0) next = atomicAdd(A.queue, 1);
    __syncthreads();
    const int q = next;
    __syncthreads();
    if (q >= A.nsolve * nitem) break;
    const int item = q / A.nsolve;
    const int s = A.order[q % A.nsolve];
    int* const ss = cut ? A.sstate + (size_t)kSolveStateInts * s : nullptr;
    const PeriodDev P = A.periods[A.pidx[s]];
    const size_t N = (size_t)P.nx * P.ny;
    if (cut && item > 0) {
      if (threadIdx.x == 0) {
        int d = ld_acquire(ss + SS_DONE), it = 0;
        while (d >= 0 && d < item && it < kItemWaitLimit) {
          __nanosleep(128);
          d = ld_acquire(ss + SS_DONE);
          ++it;
        }
        prev_done = d;
        prev_fit = ss[SS_FIT];
        prev_fst = ss[SS_FST];
      }
      __syncthreads();
      const int d = prev_done;
      if (d < 0) continue;  // the solve failed in an earlier item
      if (d < item) {       // wait limit: report and drop the solve
        solve_fail(A, P, s, ST_TIMEOUT);
        if (threadIdx.x == 0) {
          __threadfence();
          st_release(ss + SS_DONE, -1);
        }
        __syncthreads();
        continue;
      }
    }
    if (threadIdx.x == 0) sh.flag = ST_OK;
    SolveLayout L = carve(base, N);
    FwdWs fw = L.fw;
    double* grad = nullptr;
    if (cut) {
      const long long S = A.solve_cells;
      fw.tau = A.ws_solve + A.kslot[s];
      fw.T0 = A.ws_solve + S + A.kslot[s];
      grad = A.ws_solve + 2 * S + A.kslot[s];
    }
    double x0 = A.srcx[s], y0 = A.srcy[s];
    if (P.lonlat) {
      x0 = x0 / 180.0 * PI_S;
      y0 = y0 / 180.0 * PI_S;
    }
    fwd_setup(P, x0, y0, 1.0, 1.0, 10.0, fw, true, sh, grad, (size_t)A.solve_cells,
              cut && item > 0);
    if (sh.status != ST_OK) {
      const int st = sh.status;
      __syncthreads();
      solve_fail(A, P, s, st);
      if (cut && threadIdx.x == 0) {
        __threadfence();
        st_release(ss + SS_DONE, -1);
      }
      __syncthreads();
      continue;
    }
    const bool last = !cut || item == nitem - 1;
    int fst, fit;
    if (cut && item > 0 && prev_fst == ST_OK) {  // converged in an earlier item
      fst = ST_OK;
      fit = prev_fit;
    } else {
      const int it0 = cut && item > 0 ? prev_fit + 1 : 1;
      const int it1 = last ? MAXITER_UW : (item + 1) * kFp64SplitIter;
      uw_sweeps(P, fw, sh, it1, it0);
      fst = sh.status;
      fit = sh.iters;
    }
    if (!last) {
      if (threadIdx.x == 0) {
        ss[SS_FIT] = fit;
        ss[SS_FST] = fst;
        __threadfence();
        st_release(ss + SS_DONE, item + 1);
      }
      __syncthreads();
      continue;
    }
    for (size_t k = threadIdx.x; k < N; k += blockDim.x) L.T[k] = fw.tau[k] * fw.T0[k];
    if (A.fwd_updates && threadIdx.x == 0) {
      const Box b = sh.box;
      const double frozen = (double)(b.i1 - b.i0 + 1) * (b.j1 - b.j0 + 1);
      A.fwd_updates[s] = (double)fit * 4.0 * ((double)N - frozen);
    }
    __syncthreads();
    solve_tail(A, P, s, L.T, L.aw, sh, fst, fit);
    if (cut && threadIdx.x == 0) {
      __threadfence();
      st_release(ss + SS_DONE, nitem);
    }
    __syncthreads();
  }
}

void launch_batch_fp64(const BatchArgs& a, int grid, int block, cudaStream_t st) {
  k_batch_fp64<<<grid, block, 0, st>>>(a);
}

int batch_fp64_max_blocks_per_sm(int block) {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_fp64, block, 0);
  return n;
}

// ---------------------------------------------------------------------------
// Ordered reductions
// ---------------------------------------------------------------------------
__global__ void k_kernel_reduce(int nperiod, const int* plist_off, const int* plist,
                                const long long* kslot, const double* contrib, double* out,
                                const long long* goff, const int* nxs, const int* nys) {
  const int p = blockIdx.y;
  if (p >= nperiod) return;
  const long long N = (long long)nxs[p] * nys[p];
  const int s0 = plist_off[p], s1 = plist_off[p + 1];
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < N;
       k += (long long)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int q = s0; q < s1; ++q) acc = acc + contrib[kslot[plist[q]] + k];
    out[goff[p] + k] = acc;
  }
}

void launch_kernel_reduce(const PeriodDev* /*periods_host*/, int nperiod, const int* plist_off,
                          const int* plist, const long long* kslot, const double* contrib,
                          double* out, long long /*ncell*/, const long long* goff_dev,
                          const int* nx_dev, const int* ny_dev, cudaStream_t st) {
  dim3 grid(64, nperiod);
  k_kernel_reduce<<<grid, 256, 0, st>>>(nperiod, plist_off, plist, kslot, contrib, out,
                                        goff_dev, nx_dev, ny_dev);
}

// Per period and cell: the sum over the period's solves, in solve order, of
// the FP32 kernel slots of one or two fields (c1 null: one), in FP64.  The
// loads of eight solves are issued before their in-order additions, so the
// chain waits for memory once per eight solves, not once per solve.
__global__ void k_kernel_reduce_f32(int nperiod, const int* plist_off, const int* plist,
                                    const long long* kslot, const float* c0, double* o0,
                                    const float* c1, double* o1, const long long* goff,
                                    const int* nxs, const int* nys) {
  const int p = blockIdx.y;
  if (p >= nperiod) return;
  const long long N = (long long)nxs[p] * nys[p];
  const int s0 = plist_off[p], s1 = plist_off[p + 1];
  constexpr int U = 8;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < N;
       k += (long long)gridDim.x * blockDim.x) {
    double a0 = 0.0, a1 = 0.0;
    int q = s0;
    for (; q + U <= s1; q += U) {
      float v0[U], v1[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const long long off = kslot[plist[q + u]] + k;
        v0[u] = c0[off];
        v1[u] = c1 ? c1[off] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        a0 = a0 + (double)v0[u];
        a1 = a1 + (double)v1[u];
      }
    }
    for (; q < s1; ++q) {
      const long long off = kslot[plist[q]] + k;
      a0 = a0 + (double)c0[off];
      if (c1) a1 = a1 + (double)c1[off];
    }
    o0[goff[p] + k] = a0;
    if (c1) o1[goff[p] + k] = a1;
  }
}

void launch_kernel_reduce_f32(int nperiod, const int* plist_off, const int* plist,
                              const long long* kslot, const float* c0, double* o0,
                              const float* c1, double* o1, const long long* goff_dev,
                              const int* nx_dev, const int* ny_dev, cudaStream_t st) {
  dim3 grid(64, nperiod);
  k_kernel_reduce_f32<<<grid, 256, 0, st>>>(nperiod, plist_off, plist, kslot, c0, o0, c1, o1,
                                            goff_dev, nx_dev, ny_dev);
}

__global__ void k_chi_reduce(const double* chi_s, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double acc = 0.0;
    for (int s = 0; s < n; ++s) acc = acc + chi_s[s];
    *out = acc;
  }
}

void launch_chi_reduce(const double* chi_s, int nsolve, double* chi_out, cudaStream_t st) {
  k_chi_reduce<<<1, 32, 0, st>>>(chi_s, nsolve, chi_out);
}

// ---------------------------------------------------------------------------
// WENO3 sweeps (FSM_WENO3_PS_2d :344-548, FSM_WENO3_PS_multi_2d :552-761)
// ---------------------------------------------------------------------------
__device__ inline double weno_w(double u, double v) {
  const double r = (EPS14 + u * u) / (EPS14 + v * v);
  return 1.0 / (1 + 2 * (r * r));
}

__device__ inline void weno_pair(const double* tau, size_t k, size_t s, int i, int n, double h,
                                 double* p1, double* p2) {
  const double tm1 = tau[k - s], t0 = tau[k], tp1 = tau[k + s];
  if (i == 1) {
    const double tp2 = tau[k + 2 * s];
    *p1 = (t0 - tm1) / h;
    const double w2 = weno_w(t0 - 2 * tp1 + tp2, tm1 - 2 * t0 + tp1);
    *p2 = (1 - w2) * (tp1 - tm1) / 2 / h + w2 * (-3 * t0 + 4 * tp1 - tp2) / 2 / h;
  } else if (i == n - 2) {
    const double tm2 = tau[k - 2 * s];
    const double w1 = weno_w(t0 - 2 * tm1 + tm2, tp1 - 2 * t0 + tm1);
    *p1 = (1 - w1) * (tp1 - tm1) / 2 / h + w1 * (3 * t0 - 4 * tm1 + tm2) / 2 / h;
    *p2 = (tp1 - t0) / h;
  } else {
    const double tm2 = tau[k - 2 * s], tp2 = tau[k + 2 * s];
    const double w1 = weno_w(t0 - 2 * tm1 + tm2, tp1 - 2 * t0 + tm1);
    *p1 = (1.0 - w1) * (tp1 - tm1) / 2 / h + w1 * (3 * t0 - 4 * tm1 + tm2) / 2 / h;
    const double w2 = weno_w(t0 - 2 * tp1 + tp2, tm1 - 2 * t0 + tp1);
    *p2 = (1.0 - w2) * (tp1 - tm1) / 2 / h + w2 * (-3 * t0 + 4 * tp1 - tp2) / 2 / h;
  }
}

__device__ inline void weno_sweeps(const PeriodDev& P, const FwdWs& W, SolveShared& sh, int multi) {
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  const Box box = sh.box;
  double* tau = W.tau;
  double* tau_old = W.tau_old;
  const double* T0 = W.T0;
  const double* T0x = W.K;
  const double* T0y = W.K + N;
  const double dx = P.dx, dy = P.dy;
  int iter, status = ST_NOT_CONVERGED;
  for (iter = 1; iter <= MAXITER_WENO; ++iter) {
    for (size_t k = threadIdx.x; k < N; k += blockDim.x) tau_old[k] = tau[k];
    __syncthreads();
    for (int s = 0; s < 4; ++s) {
      SweepGeom g;
      g.ilo = 1; g.ihi = nx - 2; g.jlo = 1; g.jhi = ny - 2;
      sweep_dirs(s, g.xdir, g.ydir);
      const int nd = g.ndiag();
      for (int d = 0; d < nd; ++d) {
        for (int v = g.vmin(d) + (int)threadIdx.x; v <= g.vmax(d); v += blockDim.x) {
          int i, j;
          g.cell(d, v, i, j);
          if (box.has(i, j)) continue;
          const size_t k = (size_t)i + (size_t)nx * j;
          const double a = P.a[k], b = P.b[k], c = P.c[k];
          float sigx, sigy;
          if (multi) {
            sigx = (float)(sqrt(a) * T0[k]);
            sigy = (float)(sqrt(b) * T0[k]);
          } else {
            sigx = (float)sqrt(a);
            sigy = (float)sqrt(b);
          }
          const float coe = (float)(1.0 / (((double)sigx / dx) + ((double)sigy / dy)));
          double px1, px2, py1, py2;
          weno_pair(tau, k, 1, i, nx, dx, &px1, &px2);
          weno_pair(tau, k, (size_t)nx, j, ny, dy, &py1, &py2);
          double H;
          if (multi) {
            const double U = T0x[k] * tau[k] + T0[k] * (px1 + px2) / 2;
            const double V = T0y[k] * tau[k] + T0[k] * (py1 + py2) / 2;
            H = sqrt(a * (U * U) + b * (V * V) - 2 * c * U * V);
          } else {
            const double Pp = (px1 + px2) / 2, Q = (py1 + py2) / 2;
            H = sqrt(a * (Pp * Pp) + b * (Q * Q) - 2 * c * (px1 + px2) * (py1 + py2) / 4 +
                     2 * (a * T0x[k] - c * T0y[k]) * (px1 + px2) / 2 +
                     2 * (b * T0y[k] - c * T0x[k]) * (py1 + py2) / 2 + a * (T0x[k] * T0x[k]) +
                     b * (T0y[k] * T0y[k]) - 2 * c * T0x[k] * T0y[k]);
          }
          tau[k] = (double)coe * (P.fun[k] - H) +
                   (double)coe * ((double)sigx * (px2 - px1) / 2 + (double)sigy * (py2 - py1) / 2) +
                   tau[k];
        }
        __syncthreads();
      }
      // boundary extrapolation after every sweep (:502-509, :715-722)
      const int jlo = multi ? 1 : 0, jhi = multi ? ny - 1 : ny;
      for (int j = jlo + threadIdx.x; j < jhi; j += blockDim.x) {
        const size_t r = (size_t)nx * j;
        double v1 = 2 * tau[r + 1] - tau[r + 2], v2 = tau[r + 2];
        tau[r] = v1 > v2 ? v1 : v2;
        v1 = 2 * tau[r + nx - 2] - tau[r + nx - 3];
        v2 = tau[r + nx - 3];
        tau[r + nx - 1] = v1 > v2 ? v1 : v2;
      }
      __syncthreads();
      const int ilo = multi ? 1 : 0, ihi = multi ? nx - 1 : nx;
      for (int i = ilo + threadIdx.x; i < ihi; i += blockDim.x) {
        double v1 = 2 * tau[i + (size_t)nx] - tau[i + 2 * (size_t)nx], v2 = tau[i + 2 * (size_t)nx];
        tau[i] = v1 > v2 ? v1 : v2;
        v1 = 2 * tau[i + (size_t)nx * (ny - 2)] - tau[i + (size_t)nx * (ny - 3)];
        v2 = tau[i + (size_t)nx * (ny - 3)];
        tau[i + (size_t)nx * (ny - 1)] = v1 > v2 ? v1 : v2;
      }
      __syncthreads();
    }
    double l1 = 0, lm = 0;
    for (size_t k = threadIdx.x; k < N; k += blockDim.x) {
      const double d = fabs(tau[k] - tau_old[k]);
      l1 += d * dx * dy;
      lm = fmax(lm, d);
    }
    block_sum_max(l1, lm, sh.red);
    if (fabs(l1) < TOL_WENO && lm < TOL_WENO) { status = ST_OK; break; }
  }
  if (threadIdx.x == 0) {
    sh.status = status;
    sh.iters = iter > MAXITER_WENO ? MAXITER_WENO : iter;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Single-solve kernels (one block) for the drop-in symbols
// ---------------------------------------------------------------------------
// (+ one N-cell array: the cluster forward's iteration-start tau)
long long single_ws_doubles(long long N) { return batch_fp64_ws_doubles(N) + N; }

__global__ void __launch_bounds__(256) k_uw_single(PeriodDev P, double x0, double y0, double* ws,
                                                   double* T, int* si) {
  __shared__ SolveShared sh;
  const size_t N = (size_t)P.nx * P.ny;
  SolveLayout L = carve(ws, N);
  fwd_setup(P, x0, y0, 1.0, 1.0, 10.0, L.fw, true, sh);
  if (sh.status != ST_OK) {
    if (threadIdx.x == 0) { si[0] = sh.status; si[1] = 0; }
    return;
  }
  uw_sweeps(P, L.fw, sh, MAXITER_UW);
  for (size_t k = threadIdx.x; k < N; k += blockDim.x) T[k] = L.fw.tau[k] * L.fw.T0[k];
  if (threadIdx.x == 0) { si[0] = sh.status; si[1] = sh.iters; }
}

void launch_uw_single(const PeriodDev& P, double x0, double y0, double* ws, double* T,
                      int* si, cudaStream_t st) {
  k_uw_single<<<1, 256, 0, st>>>(P, x0, y0, ws, T, si);
}

// Blocks of the cluster forward: blocks 0 - 3 evaluate the two-sided cases
// 0 - 3 of the update, block 4 the one-sided cases west and east, block 5
// south and north (about 35, 14 and 14 FP64 instructions a cell).
constexpr int kUwRanks = 6;

// What one thread needs from global memory for its cell of one diagonal:
// the cell and its block's constants, loaded while the cluster barrier of
// the previous diagonal completes.
struct UwPre {
  bool on;  // a cell of this diagonal, not in the frozen box
  int i, j;
  size_t k;
  double cx, cy, t0, old;
  double ea, bx, by, iea, a, b, c, f2;  // two-sided blocks
  double ip0, ip1, t0nb0, t0nb1, dis;   // one-sided blocks (faces f0, f0 + 1)
};

__device__ __forceinline__ void uw_fetch(const PeriodDev& P, const double* __restrict__ K,
                                         const double* __restrict__ T0,
                                         const double* __restrict__ told, const Box& box,
                                         int rank, int s, int d, UwPre& p) {
  const int nx = P.nx, ny = P.ny;
  SweepGeom g;
  g.ilo = 0; g.ihi = nx - 1; g.jlo = 0; g.jhi = ny - 1;
  sweep_dirs(s, g.xdir, g.ydir);
  const int v = g.vmin(d) + (int)threadIdx.x;
  p.on = v <= g.vmax(d);
  if (!p.on) return;
  g.cell(d, v, p.i, p.j);
  p.on = !box.has(p.i, p.j);
  if (!p.on) return;
  const size_t k = (size_t)p.i + (size_t)nx * p.j;
  p.k = k;
  const double* Kc = K + k * (size_t)KC_COUNT;
  p.cx = Kc[KC_CX];
  p.cy = Kc[KC_CY];
  p.t0 = T0[k];
  p.old = (s == 3 && rank == 0) ? told[k] : 0.0;
  if (rank < 4) {
    p.ea = Kc[KC_EA + rank];
    p.bx = Kc[KC_BX + rank];
    p.by = Kc[KC_BY + rank];
    p.iea = Kc[KC_IEA + rank];
    p.a = P.a[k];
    p.b = P.b[k];
    p.c = P.c[k];
    p.f2 = P.f2[k];
  } else {
    const int f0 = rank == 4 ? 0 : 2;
    const bool lo = f0 == 0 ? p.i > 0 : p.j > 0, hi = f0 == 0 ? p.i < nx - 1 : p.j < ny - 1;
    p.ip0 = Kc[KC_IPXM + f0];
    p.ip1 = Kc[KC_IPXM + f0 + 1];
    p.t0nb0 = lo ? T0[uw_nb(f0, k, nx)] : 0.0;
    p.t0nb1 = hi ? T0[uw_nb(f0 + 1, k, nx)] : 0.0;
    p.dis = f0 == 0 ? P.disx[k] : P.disy[k];
  }
}

// Order-preserving integer key of a double (signed compare = numeric
// compare; -0 below +0): the phase-2 minimum runs on the integer pipe.
__device__ __forceinline__ long long uw_key(double x) {
  const long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}

// One plain FP64 forward solve on a cluster of kUwRanks blocks, one per SM.
//
// A call of the drop-in is one solve, a chain of anti-diagonal steps, and an
// FP64 warp instruction holds a scheduler for the same time whatever the
// number of its active lanes: one block's step costs the whole visit's FP64
// instruction sequence however the diagonal's cells are spread over warps.
// Here the visit itself is spread: each block evaluates only its cases of
// the update (one two-sided case, or two one-sided cases) for every cell of
// the diagonal and writes its candidate minimum into every block's shared
// memory; after one cluster barrier each block takes min(tau, the six
// candidates) -- the same minimum over the same roots as uw_update -- into
// its own shared copy of tau.  Every block therefore holds the same field;
// block 0 accumulates the convergence sums and broadcasts its decision, so
// all blocks run the same number of barriers.
// Candidates are double-buffered by diagonal parity: a block writes
// diagonal d+1's only after the barrier of diagonal d, which every block
// reaches after reading diagonal d-1's.  Between its arrival at a barrier
// and the wait, a thread loads the next diagonal's cell constants (global
// memory, L2-resident), so their latency hides behind the barrier.  The
// setup is shared out by chunks; block 0's iteration-start values live in
// ws beyond the single solve's layout.  One cell per thread and diagonal
// (min(nx, ny) <= 256 = blockDim.x); block 0 adds the convergence sums in
// k_uw_single's thread order, so the results equal k_uw_single's.
__global__ void __launch_bounds__(256) k_uw_cluster(PeriodDev P, double x0, double y0, double* ws,
                                                    double* T, int* si) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  extern __shared__ double uw_dyn[];
  __shared__ SolveShared sh;
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  SolveLayout L = carve(ws, N);
  fwd_setup(P, x0, y0, 1.0, 1.0, 10.0, L.fw, true, sh, nullptr, 0, false, rank, kUwRanks);
  if (sh.status != ST_OK) {  // the same in every block
    if (rank == 0 && threadIdx.x == 0) { si[0] = sh.status; si[1] = 0; }
    return;
  }
  cl.sync();  // every block's part of the setup is visible
  double* tau = uw_dyn;
  const int maxd = nx < ny ? nx : ny;
  double* cand = uw_dyn + N;  // [2][kUwRanks][maxd]
  double* told = ws + fp64_slot_doubles((long long)N);  // block 0's
  for (size_t k = threadIdx.x; k < N; k += blockDim.x) tau[k] = L.fw.tau[k];
  __syncthreads();
  const double* __restrict__ K = L.fw.K;
  const double* __restrict__ T0 = L.fw.T0;
  const Box box = sh.box;
  const double inf = __longlong_as_double(0x7ff0000000000000LL);
  const int nd = nx + ny - 1;  // diagonals per sweep
  UwPre cur, nxt;
  uw_fetch(P, K, T0, told, box, rank, 0, 0, cur);
  int iter, status = ST_NOT_CONVERGED;
  for (iter = 1; iter <= MAXITER_UW; ++iter) {
    double l1 = 0.0, linf = 0.0;
    for (int s = 0; s < 4; ++s) {
      for (int d = 0; d < nd; ++d) {
        double* const cb = cand + (size_t)(d & 1) * kUwRanks * maxd;
        const int slot = (int)threadIdx.x;  // v - vlo
        if (cur.on) {
          const size_t k = cur.k;
          const bool hw = cur.i > 0, he = cur.i < nx - 1, hs = cur.j > 0, hn = cur.j < ny - 1;
          const double tw = hw ? tau[k - 1] : 0.0, te = he ? tau[k + 1] : 0.0;
          const double ts = hs ? tau[k - nx] : 0.0, tn = hn ? tau[k + nx] : 0.0;
          const double qw = -(cur.cx * tw), qe = cur.cx * te, qs = -(cur.cy * ts),
                       qn = cur.cy * tn;
          double m = inf;
          if (rank < 4) {
            uw_two_sided_v(rank, cur.ea, cur.bx, cur.by, cur.iea, hw, he, hs, hn, qw, qe, qs, qn,
                           cur.a, cur.b, cur.c, cur.f2, m);
          } else {
            const int f0 = rank == 4 ? 0 : 2;
            uw_one_sided_v(f0, cur.ip0, cur.t0nb0, cur.dis, hw, he, hs, hn, qw, qe, qs, qn, tw,
                           te, ts, tn, cur.t0, m);
            uw_one_sided_v(f0 + 1, cur.ip1, cur.t0nb1, cur.dis, hw, he, hs, hn, qw, qe, qs, qn,
                           tw, te, ts, tn, cur.t0, m);
          }
#pragma unroll
          for (int q = 0; q < kUwRanks; ++q)
            cl.map_shared_rank(cb, q)[rank * maxd + slot] = m;
        }
        asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
        {  // the next diagonal (of the next sweep, or of the next iteration's first)
          int s2 = s, d2 = d + 1;
          if (d2 == nd) { d2 = 0; s2 = s + 1 < 4 ? s + 1 : 0; }
          uw_fetch(P, K, T0, told, box, rank, s2, d2, nxt);
        }
        asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
        if (cur.on) {
          const size_t k = cur.k;
          const double tb = tau[k];
          if (s == 0 && rank == 0) told[k] = tb;
          // min(tb, candidates): no candidate is NaN (each was taken by a
          // comparison), so the integer keys order them as the values
          long long best = uw_key(tb);
          double tn = tb;
#pragma unroll
          for (int q = 0; q < kUwRanks; ++q) {
            const double mq = cb[q * maxd + slot];
            const long long kq = uw_key(mq);
            if (kq < best) { best = kq; tn = mq; }
          }
          tau[k] = tn;
          if (s == 3 && rank == 0) {
            const double dd = fabs(tn - cur.old) * cur.t0;
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
    // block 0's decision, followed by every block
    if (rank == 0 && threadIdx.x == 0) {
      const int conv = fabs(l1) < TOL_UW && linf < TOL_UW;
#pragma unroll
      for (int q = 0; q < kUwRanks; ++q) cl.map_shared_rank(&sh.flag, q)[0] = conv;
    }
    cl.sync();
    if (sh.flag) { status = ST_OK; break; }
  }
  for (size_t k = threadIdx.x + (size_t)rank * blockDim.x; k < N;
       k += (size_t)blockDim.x * kUwRanks)
    T[k] = tau[k] * T0[k];
  if (rank == 0 && threadIdx.x == 0) {
    si[0] = status;
    si[1] = iter > MAXITER_UW ? MAXITER_UW : iter;
  }
  cl.sync();  // no block leaves while another may still address its shared memory
}

// Shared memory of k_uw_cluster: tau and the candidate buffers, at least
// 116 KB so that two of its blocks never share an SM (their FP64 pipes are
// what the cluster spreads the visit over).
static size_t uw_cluster_smem(int nx, int ny) {
  const size_t need = ((size_t)nx * ny + (size_t)2 * kUwRanks * (nx < ny ? nx : ny)) *
                      sizeof(double);
  return need < (size_t)116 * 1024 ? (size_t)116 * 1024 : need;
}

bool launch_uw_cluster(const PeriodDev& P, double x0, double y0, double* ws, double* T, int* si,
                       cudaStream_t st) {
  static const size_t max_smem = [] {
    int dev = 0, opt = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&opt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const size_t lim = (size_t)opt - sizeof(SolveShared) - 1024;
    if (cudaFuncSetAttribute(k_uw_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)lim) != cudaSuccess) {
      cudaGetLastError();
      return (size_t)0;
    }
    return lim;
  }();
  const size_t smem = uw_cluster_smem(P.nx, P.ny);
  if (smem > max_smem || (P.nx < P.ny ? P.nx : P.ny) > 256) return false;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kUwRanks);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kUwRanks;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, k_uw_cluster, P, x0, y0, ws, T, si) != cudaSuccess) {
    cudaGetLastError();  // this launch's own error: the caller takes the one-block kernel
    return false;
  }
  return true;
}

__global__ void __launch_bounds__(256) k_weno_single(PeriodDev P, double x0, double y0, int multi,
                                                     double* ws, double* T, int* si) {
  __shared__ SolveShared sh;
  const size_t N = (size_t)P.nx * P.ny;
  SolveLayout L = carve(ws, N);
  fwd_setup(P, x0, y0, 2.0, multi ? 1.0 : 0.0, multi ? 1.0 : 20.0, L.fw, false, sh);
  if (sh.status != ST_OK) {
    if (threadIdx.x == 0) { si[0] = sh.status; si[1] = 0; }
    return;
  }
  weno_sweeps(P, L.fw, sh, multi);
  for (size_t k = threadIdx.x; k < N; k += blockDim.x)
    T[k] = multi ? L.fw.tau[k] * L.fw.T0[k] : L.fw.tau[k] + L.fw.T0[k];
  if (threadIdx.x == 0) { si[0] = sh.status; si[1] = sh.iters; }
}

void launch_weno_single(const PeriodDev& P, double x0, double y0, int multi, double* ws,
                        double* T, int* si, cudaStream_t st) {
  k_weno_single<<<1, 256, 0, st>>>(P, x0, y0, multi, ws, T, si);
}

// One adjoint field swept with the field and its iteration-start copy in
// shared memory (dynamic, 2N doubles) and each thread's next cell constants
// loaded before the block barrier of the current diagonal, so that a step
// is the visit's five FP64 operations on shared operands rather than the
// latency of its global loads.  Same arithmetic, visit order, thread-to-cell
// map and reductions as adj_sweeps with one field; one cell per thread and
// diagonal (min(nx, ny) - 2 <= blockDim.x).
struct JsePre {
  bool on;
  size_t k;
  double ww, we, ws, wn, id, dl;
};

__device__ __forceinline__ void jse_fetch(const PeriodDev& P, const double* __restrict__ K,
                                          const double* __restrict__ delta, int s, int d,
                                          JsePre& p) {
  const int nx = P.nx, ny = P.ny;
  SweepGeom g;
  g.ilo = 1; g.ihi = nx - 2; g.jlo = 1; g.jhi = ny - 2;
  sweep_dirs(s, g.xdir, g.ydir);
  const int v = g.vmin(d) + (int)threadIdx.x;
  p.on = v <= g.vmax(d);
  if (!p.on) return;
  int i, j;
  g.cell(d, v, i, j);
  const size_t k = (size_t)i + (size_t)nx * j;
  p.k = k;
  const double* Kr = K + k * (size_t)KA_COUNT;
  p.ww = Kr[KA_WW];
  p.we = Kr[KA_WE];
  p.ws = Kr[KA_WS];
  p.wn = Kr[KA_WN];
  p.id = Kr[KA_ID];
  p.dl = delta[k];
}

__device__ inline void adj_sweeps_shared(const PeriodDev& P, const AdjWs& W, double* ta,
                                         double* old, SolveShared& sh, int* its, int* sts) {
  const int nx = P.nx, ny = P.ny;
  const size_t N = (size_t)nx * ny;
  const double* __restrict__ K = W.K;
  const double* __restrict__ delta = W.delta[0];
  for (size_t k = threadIdx.x; k < N; k += blockDim.x) ta[k] = W.Ta[0][k];
  __syncthreads();
  const int nd = (nx - 2) + (ny - 2) - 1;
  JsePre cur, nxt;
  jse_fetch(P, K, delta, 0, 0, cur);
  int iter, status = ST_NOT_CONVERGED;
  for (iter = 1; iter <= MAXITER_JSE; ++iter) {
    double l1 = 0, lm = 0;
    for (int s = 0; s < 4; ++s) {
      for (int d = 0; d < nd; ++d) {
        if (cur.on) {
          const size_t k = cur.k;
          const double before = ta[k];
          if (s == 0) old[k] = before;
          const double nv = cur.dl * cur.id + cur.ww * ta[k - 1] + cur.we * ta[k + 1] +
                            cur.ws * ta[k - nx] + cur.wn * ta[k + nx];
          ta[k] = nv;
          if (s == 3) {
            const double dd = fabs(nv - old[k]);
            l1 += dd;
            lm = fmax(lm, dd);
          }
        }
        int s2 = s, d2 = d + 1;
        if (d2 == nd) { d2 = 0; s2 = s + 1 < 4 ? s + 1 : 0; }
        jse_fetch(P, K, delta, s2, d2, nxt);
        __syncthreads();
        cur = nxt;
      }
    }
    block_sum_max(l1, lm, sh.red);
    l1 = l1 / (double)(nx * ny);
    if (fabs(l1) < TOL_JSE && lm < TOL_JSE) { status = ST_OK; break; }
  }
  its[0] = iter > MAXITER_JSE ? MAXITER_JSE : iter;
  sts[0] = status;
  for (size_t k = threadIdx.x; k < N; k += blockDim.x) W.Ta[0][k] = ta[k];
  __syncthreads();
}

__global__ void __launch_bounds__(256) k_jse_single(PeriodDev P, const double* T,
                                                    const double* recx, const double* recy,
                                                    const double* sadj, int nrec, double* ws,
                                                    double* Ta, int* si, int shared_field) {
  extern __shared__ double jse_dyn[];
  __shared__ SolveShared sh;
  const size_t N = (size_t)P.nx * P.ny;
  SolveLayout L = carve(ws, N);
  L.aw.T = T;
  L.aw.Ta[0] = Ta;
  for (size_t k = threadIdx.x; k < N; k += blockDim.x) L.aw.delta[0][k] = 0.0;
  __syncthreads();
  if (threadIdx.x == 0) sh.flag = adj_splat(P, L.aw.delta[0], nrec, recx, recy, sadj, 0.0);
  __syncthreads();
  if (sh.flag != ST_OK) {
    if (threadIdx.x == 0) { si[0] = sh.flag; si[1] = 0; }
    return;
  }
  adj_setup(P, L.aw, 1);
  int its[2] = {0, 0}, sts[2] = {ST_OK, ST_OK};
  if (shared_field)
    adj_sweeps_shared(P, L.aw, jse_dyn, jse_dyn + N, sh, its, sts);
  else
    adj_sweeps(P, L.aw, 1, sh, its, sts);
  if (threadIdx.x == 0) { si[0] = sts[0]; si[1] = its[0]; }
}

void launch_jse_single(const PeriodDev& P, const double* T, const double* recx,
                       const double* recy, const double* sadj, int nrec, double* ws, double* Ta,
                       int* si, cudaStream_t st) {
  static const size_t max_smem = [] {
    int dev = 0, opt = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&opt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const size_t lim = (size_t)opt - sizeof(SolveShared) - 1024;
    if (cudaFuncSetAttribute(k_jse_single, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)lim) != cudaSuccess) {
      cudaGetLastError();
      return (size_t)0;
    }
    return lim;
  }();
  // the field and its iteration-start copy in shared memory when they fit
  const size_t smem = (size_t)2 * P.nx * P.ny * sizeof(double);
  const bool shared = smem <= max_smem && (P.nx < P.ny ? P.nx : P.ny) - 2 <= 256;
  k_jse_single<<<1, 256, shared ? smem : 0, st>>>(P, T, recx, recy, sadj, nrec, ws, Ta, si,
                                                   shared ? 1 : 0);
}

__global__ void k_mask_single(PeriodDev P, double* tab, double x0, double y0) {
  apply_mask(P, tab, x0, y0);
}

void launch_mask_single(const PeriodDev& P, double* tab, double x0, double y0, cudaStream_t st) {
  k_mask_single<<<1, 256, 0, st>>>(P, tab, x0, y0);
}

__global__ void k_interp(PeriodDev P, const double* T, int nrec, const double* recx,
                         const double* recy, double* out, int* status) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrec) return;
  double v = 0;
  if (!interp2(P.xdeg, P.nx, P.ydeg, P.ny, T, recx[r], recy[r], &v)) atomicExch(status, ST_BAD_ARG);
  out[r] = v;
}

void launch_interp(const PeriodDev& P, const double* T, int nrec, const double* recx,
                   const double* recy, double* out, int* status, cudaStream_t st) {
  if (nrec <= 0) return;
  k_interp<<<(nrec + 127) / 128, 128, 0, st>>>(P, T, nrec, recx, recy, out, status);
}

}  // namespace sgb
