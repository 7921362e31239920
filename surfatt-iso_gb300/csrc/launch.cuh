// launch.cuh -- one gradient evaluation on device-resident buffers: launch
// configuration (block size, shared memory, resident blocks) and the kernel
// sequence (batched solve kernel, ordered per-period kernel sums, misfit
// sum).  Used by the engine and by the serving loop.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "kernels.cuh"

namespace sgb {

// Host-side shape of an evaluation (what the launch configuration needs).
// Team classes: solves whose grids need t warps of the row kernel (t = 1 ..
// kTeamMaxRows / 128) form class t.
constexpr int kTeamClasses = kTeamMaxRows / 128;

struct EvalShape {
  int nperiod = 0, nsolve = 0, npath = 0;
  long long ncell = 0, max_cells = 0, max_pitched = 0;
  int max_nx = 0, max_ny = 0, max_diag = 0;
  long long solve_cells = 0;  // sum over the solves of their grids' cells (with pidx)
  // Solves per team class and the class's tallest grid, counted when
  // from_grids is given the solves' period indices (else all zero: the
  // evaluation is launched as one class).
  int team_count[kTeamClasses] = {}, team_max_ny[kTeamClasses] = {};
  void from_grids(const int* nx, const int* ny, const long long* goff, int np, int ns, int npth,
                  const int* pidx = nullptr);
};

// Sort key that makes the team classes contiguous in a processing order,
// the class of the tallest grids first (larger key first).
int team_class_key(int ny);

// Device pointers of an evaluation (inputs, outputs, per-period reduction
// lists).  `args` is the solve kernel's argument block without workspace.
struct EvalDev {
  BatchArgs args;
  const int* plist_off;   // per-period solve lists (work-list order)
  const int* plist;
  const long long* goff;
  const int* nx;
  const int* ny;
  double* chi_total;      // 1 double
  double* adj_s;          // ncell
  double* adj_density;    // ncell
};

// Solve kernels: plain FP64 (one block per solve), FP32 one block per solve
// (any grid), FP32 one warp (or a team of warps) per solve, lanes owning
// the rows (grids of at most 512 rows and 4096 columns).
enum KernelKind { KK_FP64 = 0, KK_FP32_BLOCK = 1, KK_FP32_WARP = 2 };

// A solve-kernel choice; -1 fields are picked automatically.  `variant`
// indexes the warp kernel's operand-prefetch / register-cap variants.
struct KernelChoice {
  int kind = -1, variant = -1;
};

struct LaunchPlan {
  int kind = KK_FP64;
  int grid = 0, block = 0, per_sm = 0, smem_tau = 0, bands = 0, pf = 1;
  int slots_per_block = 1;   // solves resident per block (warps for KK_FP32_WARP)
  bool cut = false;          // solves cut into work items: one workspace slot per solve
  size_t smem = 0;
  long long ws_doubles = 0;  // per resident solve
  long long solve_doubles = 0;  // KK_FP64 with items: per-solve tau arrays (all solves)
  // KK_FP32_WARP on a batch of several team classes: one launch per class
  // (largest team first), each over its contiguous part of the processing
  // order, with its own queue counter, band count and grid.  classes == 1:
  // one launch over every solve.
  int classes = 1;
  int class_solves[kTeamClasses] = {}, class_off[kTeamClasses] = {};
  int class_grid[kTeamClasses] = {}, class_bands[kTeamClasses] = {};
};

// Launch configuration for `prec` (0 FP64, 1 FP32) on `device`; grid capped
// at `max_grid` (0 = resident capacity of the device).  Returns ST_BAD_ARG
// when a grid's diagonal exceeds the FP32 kernel's block limit.
// `force` selects a kernel variant, as the autotuner does when it times the
// candidates.
int plan_evaluation(const EvalShape& sh, int prec, int device, int max_grid, LaunchPlan* plan,
                    const KernelChoice& force = KernelChoice());

// Doubles of workspace an evaluation of `nsolve` solves needs under `plan`
// (slots, then the per-solve state records of a cut evaluation).
long long plan_ws_doubles(const LaunchPlan& plan, int nsolve);

// Kernel variants the autotuner times for an evaluation of this shape.
std::vector<KernelChoice> plan_candidates(const EvalShape& sh, int prec);

// Streams and events for the class launches of a split plan: class c > 0
// runs on side[c - 1], forked from and joined back into the main stream by
// fork / join[c - 1] (events without timing).
struct ClassStreams {
  cudaStream_t side[kTeamClasses - 1] = {};
  cudaEvent_t fork = nullptr, join[kTeamClasses - 1] = {};
  int create();   // ST_OK or ST_CUDA_ERROR
  void destroy();
};

// Enqueue the evaluation on `st`: queue reset, tt_fwd reset, solve kernel(s),
// per-period reductions (modes 2, 3) and the misfit sum.  `ws` must hold
// plan_ws_doubles(plan, nsolve) doubles; `queue` plan.classes ints.  The
// class launches of a split plan run concurrently on `cs` (one after
// another on `st` when null).  Records ev_k0/ev_k1 around the solve
// kernels when given.  Returns the number of kernel launches, or a negative
// status.
int enqueue_evaluation(const EvalShape& sh, const EvalDev& dev, const LaunchPlan& plan, int mode,
                       int prec, double* ws, int* queue, cudaStream_t st, cudaEvent_t ev_k0,
                       cudaEvent_t ev_k1, const ClassStreams* cs = nullptr);

}  // namespace sgb
