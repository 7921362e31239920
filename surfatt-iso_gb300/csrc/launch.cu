// launch.cu -- launch configuration and kernel sequence of one gradient
// evaluation (shared by the engine and the serving loop).
#include <algorithm>

#include "launch.cuh"

namespace sgb {

int team_class_key(int ny) { return std::min(fp32w_team(ny), kTeamClasses + 1); }

void EvalShape::from_grids(const int* nxs, const int* nys, const long long* goffs, int np, int ns,
                           int npth, const int* pidx) {
  nperiod = np;
  nsolve = ns;
  npath = npth;
  ncell = max_cells = max_pitched = 0;
  max_nx = max_ny = max_diag = 0;
  for (int p = 0; p < np; ++p) {
    const long long N = (long long)nxs[p] * nys[p];
    ncell = std::max(ncell, goffs[p] + N);
    max_cells = std::max(max_cells, N);
    max_nx = std::max(max_nx, nxs[p]);
    max_ny = std::max(max_ny, nys[p]);
    max_diag = std::max(max_diag, std::min(nxs[p], nys[p]));
    max_pitched = std::max(max_pitched, (long long)batch_fp32_pitch(nxs[p]) * nys[p]);
  }
  for (int c = 0; c < kTeamClasses; ++c) team_count[c] = team_max_ny[c] = 0;
  solve_cells = 0;
  if (pidx)
    for (int s = 0; s < ns; ++s) {
      solve_cells += (long long)nxs[pidx[s]] * nys[pidx[s]];
      const int y = nys[pidx[s]], c = team_class_key(y) - 1;
      if (c >= kTeamClasses) continue;  // taller than any team
      ++team_count[c];
      team_max_ny[c] = std::max(team_max_ny[c], y);
    }
}

std::vector<KernelChoice> plan_candidates(const EvalShape& sh, int prec) {
  std::vector<KernelChoice> c;
  if (prec == 0) {
    c.push_back({KK_FP64, 0});  // work items
    c.push_back({KK_FP64, 1});  // whole solves
    return c;
  }
  // (the strip variants differ from 0 and 1 only on grids of more than 128 rows)
  if (sh.max_ny <= kTeamMaxRows && sh.max_nx <= kWarpMaxCols)
    for (int v = 0; v < fp32w_variant_count(); ++v)
      if (!fp32w_variant_strips(v) || sh.max_ny > 128) c.push_back({KK_FP32_WARP, v});
  if (sh.max_diag <= kFp32MaxThreads) c.push_back({KK_FP32_BLOCK, 0});
  return c;
}

int plan_evaluation(const EvalShape& sh, int prec, int device, int max_grid, LaunchPlan* plan,
                    const KernelChoice& force) {
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return ST_CUDA_ERROR;
  LaunchPlan p;
  if (prec == 0) {
    // variant 0: solves cut into work items (per-solve tau arrays, needs the
    // solves' cells); variant 1: whole solves
    p.kind = KK_FP64;
    p.block = 128;
    p.per_sm = batch_fp64_max_blocks_per_sm(p.block);
    p.ws_doubles = batch_fp64_ws_doubles(sh.max_cells);
    p.pf = force.variant == 1 ? 1 : 0;
    p.cut = p.pf == 0 && sh.solve_cells > 0;
    if (!p.cut) p.pf = 1;
    p.solve_doubles = p.cut ? 4 * sh.solve_cells : 0;  // tau, T0, T0x, T0y per solve
  } else if (force.kind == KK_FP32_WARP &&
             !(sh.max_ny <= kTeamMaxRows && sh.max_nx <= kWarpMaxCols)) {
    return ST_BAD_ARG;  // the row kernel holds 512 rows
  } else if (force.kind != KK_FP32_BLOCK && sh.max_ny <= kTeamMaxRows &&
             sh.max_nx <= kWarpMaxCols) {
    // one warp (a team of warps above 128 rows) per solve, lanes own the rows
    // automatic: the row-per-lane kernel (the faster on the measured shapes)
    p.kind = KK_FP32_WARP;
    p.slots_per_block = 1;
    p.bands = fp32w_bands(sh.max_ny);
    // automatic: work items, grids of more than 128 rows in strips (the
    // faster on every measured batch of tall grids and in the serving loop)
    p.pf = force.variant >= 0 && force.variant < fp32w_variant_count()
               ? force.variant
               : (sh.max_ny > 128 ? 4 : 0);
    p.block = fp32w_block(p.bands, p.pf);
    p.per_sm = batch_fp32w_max_blocks_per_sm(p.bands, p.pf);
    p.ws_doubles = batch_fp32w_ws_doubles(sh.max_cells);
    p.cut = fp32w_variant_items(p.pf);
  } else {
    // one block per solve, one thread per cell of the longest anti-diagonal
    if (sh.max_diag > kFp32MaxThreads) return ST_BAD_ARG;
    p.kind = KK_FP32_BLOCK;
    p.pf = 0;
    p.block = std::max(32, (sh.max_diag + 31) / 32 * 32);
    p.smem = batch_fp32_smem_bytes(sh.max_pitched, sh.max_nx, &p.smem_tau);
    p.per_sm = batch_fp32_max_blocks_per_sm(p.block, p.smem, p.smem_tau);
    p.ws_doubles = batch_fp32_ws_doubles(sh.max_cells);
  }
  if (p.per_sm < 1) p.per_sm = 1;
  // Resident units: one per work item, except for the strip variants' items,
  // which get one warp per solve: a solve's items then run as soon as its
  // previous item ends (its two adjoint fields side by side), and no warp
  // holds a slot waiting for a forward another warp has only begun -- slots
  // the other team classes' launches need.
  const int units_per_solve =
      p.cut ? (p.kind == KK_FP64 ? kFp64Items
                                 : (fp32w_variant_strips(p.pf) ? 1 : fp32w_items_for_mode(3)))
            : 1;
  auto grid_for = [&](int per_sm, int nsolve) {
    int g = nsm * std::max(1, per_sm);
    if (max_grid > 0) g = std::min(g, max_grid);
    const int need = (std::max(1, nsolve) * units_per_solve + p.slots_per_block - 1) /
                     p.slots_per_block;
    return std::max(1, std::min(g, need));
  };
  p.grid = grid_for(p.per_sm, sh.nsolve);
  // several team classes: one launch per class (the processing order holds
  // the classes contiguously, the largest team first)
  int nonempty = 0, counted = 0;
  for (int c = 0; c < kTeamClasses; ++c) {
    nonempty += sh.team_count[c] > 0;
    counted += sh.team_count[c];
  }
  if (p.kind == KK_FP32_WARP && nonempty == 1 && counted == sh.nsolve) {
    // one class: the team of its tallest grid (periods without solves, e.g.
    // a work list over some of a model's periods, do not widen it)
    for (int c = 0; c < kTeamClasses; ++c)
      if (sh.team_count[c] > 0) {
        p.bands = fp32w_bands(sh.team_max_ny[c]);
        p.block = fp32w_block(p.bands, p.pf);
        p.per_sm = std::max(1, batch_fp32w_max_blocks_per_sm(p.bands, p.pf));
        p.grid = grid_for(p.per_sm, sh.nsolve);
      }
  }
  if (p.kind == KK_FP32_WARP && nonempty > 1 && counted == sh.nsolve) {
    p.classes = 0;
    p.grid = 0;
    int off = 0;
    for (int c = kTeamClasses - 1; c >= 0; --c) {
      if (sh.team_count[c] == 0) continue;
      const int k = p.classes++;
      p.class_solves[k] = sh.team_count[c];
      p.class_off[k] = off;
      p.class_bands[k] = fp32w_bands(sh.team_max_ny[c]);
      p.class_grid[k] =
          grid_for(batch_fp32w_max_blocks_per_sm(p.class_bands[k], p.pf), sh.team_count[c]);
      p.grid += p.class_grid[k];
      off += sh.team_count[c];
    }
  }
  *plan = p;
  return ST_OK;
}

long long plan_ws_doubles(const LaunchPlan& plan, int nsolve) {
  const long long n = std::max(1, nsolve);
  const long long state = plan.cut ? (n * kSolveStateInts + 1) / 2 : 0;
  if (plan.kind == KK_FP64 && plan.cut)  // block slots, per-solve tau, state
    return (long long)plan.grid * plan.ws_doubles + plan.solve_doubles + state;
  // (a split plan's grid is the sum of its class grids: disjoint slots)
  const long long slots = plan.cut ? n : (long long)plan.grid * plan.slots_per_block;
  return slots * plan.ws_doubles + state;
}

int ClassStreams::create() {
  for (int i = 0; i < kTeamClasses - 1; ++i)
    if (cudaStreamCreateWithFlags(&side[i], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&join[i], cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      return ST_CUDA_ERROR;
    }
  if (cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    return ST_CUDA_ERROR;
  }
  return ST_OK;
}

void ClassStreams::destroy() {
  for (int i = 0; i < kTeamClasses - 1; ++i) {
    if (side[i]) cudaStreamDestroy(side[i]);
    if (join[i]) cudaEventDestroy(join[i]);
    side[i] = nullptr;
    join[i] = nullptr;
  }
  if (fork) cudaEventDestroy(fork);
  fork = nullptr;
}

int enqueue_evaluation(const EvalShape& sh, const EvalDev& dev, const LaunchPlan& plan, int mode,
                       int prec, double* ws, int* queue, cudaStream_t st, cudaEvent_t ev_k0,
                       cudaEvent_t ev_k1, const ClassStreams* cs) {
  BatchArgs A = dev.args;
  A.mode = mode;
  A.ws = ws;
  A.ws_doubles = plan.ws_doubles;
  A.queue = queue;
  A.block = plan.block;
  A.max_nx = sh.max_nx;
  A.smem_tau = plan.smem_tau;
  A.smem_bytes = plan.smem;
  A.items = 1;
  A.sstate = nullptr;
  if (plan.kind == KK_FP32_WARP && plan.cut) {
    const long long n = std::max(1, sh.nsolve);
    A.fwd_items = fp32w_fwd_items(plan.pf, plan.bands);
    A.adj_parts = fp32w_adj_parts(plan.pf);
    A.items = A.fwd_items + (mode == 3 ? 2 : (mode == 2 ? 1 : 0)) * A.adj_parts;
    A.sstate = reinterpret_cast<int*>(ws + n * plan.ws_doubles);
    if (cudaMemsetAsync(A.sstate, 0, (size_t)n * kSolveStateInts * sizeof(int), st) != cudaSuccess)
      return -ST_CUDA_ERROR;
  }
  if (plan.kind == KK_FP64 && plan.cut) {
    const long long n = std::max(1, sh.nsolve);
    A.items = kFp64Items;
    A.ws_solve = ws + (long long)plan.grid * plan.ws_doubles;
    A.solve_cells = plan.solve_doubles / 4;
    A.sstate = reinterpret_cast<int*>(A.ws_solve + plan.solve_doubles);
    if (cudaMemsetAsync(A.sstate, 0, (size_t)n * kSolveStateInts * sizeof(int), st) != cudaSuccess)
      return -ST_CUDA_ERROR;
  }
  int launches = 0;
  if (cudaMemsetAsync(queue, 0, std::max(1, plan.classes) * sizeof(int), st) != cudaSuccess)
    return -ST_CUDA_ERROR;
  if (A.phase_cycles &&
      cudaMemsetAsync(A.phase_cycles, 0, PH_COUNT * sizeof(unsigned long long), st) != cudaSuccess)
    return -ST_CUDA_ERROR;
  if (sh.npath > 0 &&
      cudaMemsetAsync(A.tt_fwd, 0, (size_t)sh.npath * sizeof(double), st) != cudaSuccess)
    return -ST_CUDA_ERROR;
  if (A.adj_updates && sh.nsolve > 0 &&
      cudaMemsetAsync(A.adj_updates, 0, (size_t)sh.nsolve * sizeof(double), st) != cudaSuccess)
    return -ST_CUDA_ERROR;
  // Inside a stream capture the timing events become event-record nodes of
  // the graph (recorded at every replay).
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(st, &cap);
  const unsigned ev_flags =
      cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
  if (ev_k0) cudaEventRecordWithFlags(ev_k0, st, ev_flags);
  (void)prec;
  if (sh.nsolve > 0 && plan.classes > 1) {
    // class k > 0 on side stream k - 1 (forked after the resets above), the
    // largest team's class on `st`, launched first
    if (cs && cudaEventRecord(cs->fork, st) != cudaSuccess) return -ST_CUDA_ERROR;
    long long slot0 = 0;
    for (int k = 0; k < plan.classes; ++k) {
      BatchArgs C = A;
      C.order = A.order + plan.class_off[k];
      C.nsolve = plan.class_solves[k];
      C.queue = queue + k;
      if (plan.cut && plan.kind == KK_FP32_WARP) {  // the class's own forward items
        C.fwd_items = fp32w_fwd_items(plan.pf, plan.class_bands[k]);
        C.items = C.fwd_items + (mode == 3 ? 2 : (mode == 2 ? 1 : 0)) * C.adj_parts;
      }
      if (!plan.cut) C.ws = ws + slot0 * plan.ws_doubles;  // disjoint block slots
      slot0 += plan.class_grid[k];
      cudaStream_t sk = st;
      if (cs && k > 0) {
        sk = cs->side[k - 1];
        if (cudaStreamWaitEvent(sk, cs->fork, 0) != cudaSuccess) return -ST_CUDA_ERROR;
      }
      launch_batch_fp32w(C, plan.class_grid[k], plan.class_bands[k], plan.pf, sk);
      ++launches;
      if (cs && k > 0 && (cudaEventRecord(cs->join[k - 1], sk) != cudaSuccess ||
                          cudaStreamWaitEvent(st, cs->join[k - 1], 0) != cudaSuccess))
        return -ST_CUDA_ERROR;
    }
  } else if (sh.nsolve > 0) {
    if (plan.kind == KK_FP64) launch_batch_fp64(A, plan.grid, plan.block, st);
    else if (plan.kind == KK_FP32_BLOCK) launch_batch_fp32(A, plan.grid, plan.block, st);
    else if (plan.kind == KK_FP32_WARP) launch_batch_fp32w(A, plan.grid, plan.bands, plan.pf, st);
    ++launches;
  }
  if (ev_k1) cudaEventRecordWithFlags(ev_k1, st, ev_flags);
  if (mode >= 2) {
    const int nf = mode == 3 ? 2 : 1;
    if (plan.kind == KK_FP32_WARP) {  // both fields in one pass
      launch_kernel_reduce_f32(sh.nperiod, dev.plist_off, dev.plist, A.kslot,
                               reinterpret_cast<const float*>(A.kcontrib), dev.adj_s,
                               nf == 2 ? reinterpret_cast<const float*>(A.kcontrib_den) : nullptr,
                               nf == 2 ? dev.adj_density : nullptr, dev.goff, dev.nx, dev.ny, st);
      ++launches;
    } else {
      for (int f = 0; f < nf; ++f) {
        double* kc = f == 0 ? A.kcontrib : A.kcontrib_den;
        double* out = f == 0 ? dev.adj_s : dev.adj_density;
        launch_kernel_reduce(nullptr, sh.nperiod, dev.plist_off, dev.plist, A.kslot, kc, out,
                             sh.ncell, dev.goff, dev.nx, dev.ny, st);
        ++launches;
      }
    }
  }
  launch_chi_reduce(A.chi, sh.nsolve, dev.chi_total, st);
  ++launches;
  if (cudaGetLastError() != cudaSuccess) return -ST_CUDA_ERROR;
  return launches;
}

}  // namespace sgb
