// kernels.cuh -- launch interface between the C ABI (capi.cu) and the device
// code (kernels.cu, kernels_fp32.cu).
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace sgb {

// Inputs of the per-period precompute.  Either (vel, m11, m12, m22) from the
// measurement layer -- spha = m11, sphb = m22, sphc = -m12, fun = 1./vel
// (src/measadj.f90:66-70) -- or the solver's own (spha, sphb, sphc, fun).
struct PrepIn {
  int nx, ny, lonlat;
  const double* xdeg;  // caller's coordinates (nx), degrees for lon/lat
  const double* ydeg;
  const double* A;     // m11 or spha
  const double* B;     // m22 or sphb
  const double* C;     // m12 (negated) or sphc
  const double* V;     // vel (inverted) or fun
  int from_model;      // 1: (vel, m11, m12, m22); 0: (fun, spha, sphb, sphc)
};

// Outputs (device, N per field, nx/ny per axis) -- referenced by PeriodDev.
struct PrepOut {
  double *xs, *ys, *cosy, *siny, *a, *b, *c, *fun, *f2, *disx, *disy;
  float* f32;   // optional (6N): FP32 a, b, c, fun**2, disx, disy
  double* isv;  // optional (2N): 1/svel**2, 1/svel**3 (model inputs only)
  float4* p4a;  // optional (2N): cell k's 32-byte record at 2k: {a, b, c, fun**2}
  float4* p4b;  // optional, = p4a + 1: {disx, disy, 1/svel**2, 1/svel**3} at 2k
};

// Batched evaluation arguments (all device pointers).
struct BatchArgs {
  const PeriodDev* periods;
  int nsolve;
  const int* order;        // solve processing order (cost-descending)
  const int* pidx;
  const double* srcx;
  const double* srcy;
  const int* rec_off;
  const int* nrec;
  const double* recx;
  const double* recy;
  const double* tt;
  const double* weight;
  const int* path;
  const long long* kslot;  // per solve: cell offset of its kernel contribution slot
  int mode;                // 0 forward, 2 tomo2d, 3 tomo (density too)
  // outputs
  double* tekio;           // per receiver
  double* wgt_eff;         // per receiver, weight after outlier zeroing
  double* tt_fwd;          // per path
  double* chi;             // per solve
  double* kcontrib;        // adj/svel^k slots (sum of N over solves)
  double* kcontrib_den;    // density slots (mode 3)
  int* status;
  int* fwd_iters;
  int* adj_iters;
  double* fwd_updates;     // per solve: forward cell visits (for the roofline)
  double* adj_updates;
  double* Tout;            // optional: per-solve travel-time field (kslot layout) or null
  // workspace
  double* ws;              // slots of ws_doubles each
  long long ws_doubles;
  double* ws_solve = nullptr;  // FP64 kernel with items: per-solve tau, T0, T0x, T0y planes
  long long solve_cells = 0;   // cells of one plane (the solves' kslot total)
  int* queue;              // work counter (zeroed before launch)
  int block;               // threads per block (for info)
  int max_nx;              // largest nx over periods (shared-memory column arrays)
  int smem_tau;            // FP32 kernel: 1 = tau / Ta in shared memory
  size_t smem_bytes;       // FP32 kernel: dynamic shared memory per block
  unsigned long long* phase_cycles = nullptr;  // optional: SM cycles per solve phase, summed
  int items = 1;           // FP32 warp kernel: items per solve (1: whole solves)
  int fwd_items = 0;       // FP32 warp kernel with items: forward items (0: the default)
  int adj_parts = 0;       // FP32 warp kernel with items: items per adjoint field (0: one)
  int* sstate = nullptr;   // FP32 warp kernel with items > 1: per-solve state records
  // Test hooks of the bounded item wait (FP32 warp kernel with items; off by
  // default): the first item of solve hold_solve (>= 0) is skipped without
  // being marked done, so the solve's next item waits until the poll limit
  // runs out; item_wait_limit > 0 replaces that solve's limit (every other
  // solve keeps the production limit).
  int item_wait_limit = 0;
  int hold_solve = -1;
};

// Solve phases timed when BatchArgs::phase_cycles is set (FP32 warp kernel).
enum SolvePhase {
  PH_SETUP = 0,     // source cell, frozen box, T0 field
  PH_FWD = 1,       // forward sweeps
  PH_RECV = 2,      // receiver times, misfit, outlier weights
  PH_ADJ_SETUP = 3, // adjoint coefficients and sources
  PH_ADJ = 4,       // adjoint sweeps
  PH_SLOT = 5,      // mask and kernel slot
  PH_COUNT = 6
};

void launch_prep(const PrepIn& in, const PrepOut& out, cudaStream_t st);
// The same for np periods, in as few launches as the parameter table allows.
void launch_prep_batch(const PrepIn* in, const PrepOut* out, int np, cudaStream_t st);
// Largest grid the single-warp form of the row kernel takes; its warp
// teams take up to kTeamMaxRows.
constexpr int kWarpMaxRows = 128;
constexpr int kWarpMaxCols = 4096;
constexpr int kTeamMaxRows = 512;
int fp32w_team(int max_ny);
void launch_batch_fp64(const BatchArgs& a, int grid, int block, cudaStream_t st);
void launch_batch_fp32(const BatchArgs& a, int grid, int block, cudaStream_t st);
int batch_fp64_max_blocks_per_sm(int block);
int batch_fp32_max_blocks_per_sm(int block, size_t smem_bytes, int smem_tau);
// Dynamic shared memory of the FP32 kernel: the column cos/sin arrays, plus
// tau when every grid (pitched: pitch*ny cells) fits; *tau_resident says which.
size_t batch_fp32_smem_bytes(long long max_pitched_cells, int max_nx, int* tau_resident);
int batch_fp32_pitch(int nx);
constexpr int kFp32MaxThreads = 512;
// workspace doubles per solve slot for a grid of N cells
long long batch_fp64_ws_doubles(long long N);
long long batch_fp32_ws_doubles(long long N);

// Ordered per-period kernel sum: out[goff_p + k] = sum over the solves of
// period p, in work-list order, of contrib[kslot_s + k] (src/acqui.f90:314-315).
void launch_kernel_reduce(const PeriodDev* periods_host, int nperiod, const int* plist_off,
                          const int* plist, const long long* kslot, const double* contrib,
                          double* out, long long ncell, const long long* goff_dev,
                          const int* nx_dev, const int* ny_dev, cudaStream_t st);
// Same with FP32 per-solve slots, summed in FP64.
void launch_kernel_reduce_f32(int nperiod, const int* plist_off, const int* plist,
                              const long long* kslot, const float* c0, double* o0,
                              const float* c1, double* o1, const long long* goff_dev,
                              const int* nx_dev, const int* ny_dev, cudaStream_t st);
// Warp-per-solve FP32 kernel (grids of at most 32*bands rows), one warp per
// block; `variant` < fp32w_variant_count() selects prefetch and register cap.
void launch_batch_fp32w(const BatchArgs& a, int grid, int bands, int variant, cudaStream_t st);
int batch_fp32w_max_blocks_per_sm(int bands, int variant);
int fp32w_variant_count();
// Whether a variant cuts solves into work items (one workspace slot per
// solve), and the items per solve of an evaluation mode.
bool fp32w_variant_items(int variant);
// Variants that sweep grids of more than 128 rows in strips by one warp.
bool fp32w_variant_strips(int variant);
// Threads per block of the row kernel for `bands` bands.
int fp32w_block(int bands, int variant);
int fp32w_items_for_mode(int mode);
// Forward items per solve of a variant with items on grids of `bands` bands
// (the rest: the adjoint fields' parts): strips keep each forward whole.
int fp32w_fwd_items(int variant, int bands);
// Items per adjoint field of a variant with items (iteration ranges).
int fp32w_adj_parts(int variant);
constexpr int kSolveStateInts = 11;
// Per-solve state record (ints) of a solve cut into items: items done (-1:
// failed), forward iterations, forward status, running status, adjoint
// iterations of field 0.
// (FP32 row kernel: the adjoint items' per-field iterations and statuses,
// the count of fields finished and each field's parts done)
enum SolveStateSlot { SS_DONE = 0, SS_FIT, SS_FST, SS_ST, SS_ITS0, SS_ITS1, SS_AST0, SS_AST1,
                      SS_ADJ, SS_AD0, SS_AD1 };
// Bounded wait for a solve's previous item (polls, each followed by a short
// sleep).
constexpr int kItemWaitLimit = 1 << 24;
// Release / acquire of a solve's state record between the warps or blocks
// that run its consecutive items.
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Plain FP64 kernel cut into work items (BatchArgs::items = kFp64Items):
// items 0 .. kFp64Items - 2 run kFp64SplitIter forward iterations each, the
// last runs the forward sweeps to convergence and the rest of the solve.
// (measured on the 1280-solve, 120 x 120 evaluation: 207 - 210 ms, against
// 209 - 212 ms with four to six one-iteration items)
constexpr int kFp64Items = 3;
constexpr int kFp64SplitIter = 2;
long long batch_fp32w_ws_doubles(long long N);
int fp32w_bands(int max_ny);
// chi = sum of per-solve misfits in work-list order (src/acqui.f90:135)
void launch_chi_reduce(const double* chi_s, int nsolve, double* chi_out, cudaStream_t st);

// Single-solve kernels of the drop-in symbols (one block).
void launch_uw_single(const PeriodDev& P, double x0, double y0, double* ws, double* T,
                      int* status_iters, cudaStream_t st);
// The same solve on a cluster of six blocks (one per SM), each evaluating
// its share of the update's cases; false (nothing launched) when the grid's
// tau does not fit one block's shared memory or the cluster cannot be
// launched.
bool launch_uw_cluster(const PeriodDev& P, double x0, double y0, double* ws, double* T,
                       int* status_iters, cudaStream_t st);
void launch_weno_single(const PeriodDev& P, double x0, double y0, int multiplicative, double* ws,
                        double* T, int* status_iters, cudaStream_t st);
void launch_jse_single(const PeriodDev& P, const double* T, const double* recx,
                       const double* recy, const double* sadj, int nrec, double* ws, double* Ta,
                       int* status_iters, cudaStream_t st);
void launch_mask_single(const PeriodDev& P, double* tab, double x0, double y0, cudaStream_t st);
void launch_interp(const PeriodDev& P, const double* T, int nrec, const double* recx,
                   const double* recy, double* out, int* status, cudaStream_t st);
long long single_ws_doubles(long long N);

}  // namespace sgb
