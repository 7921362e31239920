"""Work-list sharding over ranks (one GPU per rank).

The reference splits its (period, source) work list into contiguous blocks,
one per MPI rank (scatter_all_i, src/shared/parallel.f90:1877-1903,
src/src_rec.f90:368), and sums the per-period kernels, the misfit and the
synthetic-time table to rank 0 (MPI_Reduce, src/acqui.f90:152-160,
src/tomo2d.f90:196-200).  Each rank here evaluates its shard on its own GPU,
then one sum-reduction of (adj_s, adj_density, tt_fwd, chi) -- the path's
only exchange step.

Two splits:
  * ``scatter_all_i``: the reference's count split (equal numbers of solves
    per rank, contiguous blocks);
  * ``split_by_cost``: solves weighted by their predicted cost (grid cells x
    sweep iterations), assigned longest first to the least-loaded rank, each
    rank keeping its solves in work-list order.  On work lists whose grids
    differ between periods (64^2 ... 384^2 in one evaluation) a count split
    gives one rank all the large grids; the cost split does not.
"""
import numpy as np

# Sweep iterations of a point-source solve when no previous evaluation is at
# hand (forward: 4.5 - 5 on the measured workloads; adjoint: 2.5 - 3).
FWD_ITERS_NOMINAL = 5.0
ADJ_ITERS_NOMINAL = 3.0
# Cost of one adjoint iteration relative to one forward iteration of the
# same grid on the GPU (per-phase SM cycles of the FP32 solve kernel on a
# 120 x 120 grid: 4.04 M cycles per forward iteration, 1.99 M per adjoint
# iteration of one field).
ADJ_WEIGHT = 0.5


def scatter_all_i(countval, size, rank):
    """1-based inclusive (istart, iend) of `rank`'s block; empty is (1, 0)."""
    if countval < size:
        return (rank + 1, rank + 1) if rank < countval else (1, 0)
    count, remainder = divmod(countval, size)
    if rank < remainder:
        istart = rank * (count + 1) + 1
        return istart, istart + count
    istart = rank * count + remainder + 1
    return istart, istart + count - 1


def solve_costs(pb, fwd_iters=None, adj_iters=None):
    """Predicted cost of every solve of `pb`: its grid's cells x (forward
    iterations + ADJ_WEIGHT x adjoint iterations x adjoint fields).  The
    iterations are per-solve arrays from an earlier evaluation of the same
    work list (an inversion's previous gradient) when given, else nominal."""
    p = np.asarray(pb.pidx)
    cells = (np.asarray(pb.nx, np.float64) * np.asarray(pb.ny, np.float64))[p]
    nf = 2 if pb.mode == 3 else (1 if pb.mode == 2 else 0)
    fi = np.full(len(p), FWD_ITERS_NOMINAL) if fwd_iters is None else \
        np.maximum(np.asarray(fwd_iters, np.float64), 1.0)
    ai = np.full(len(p), ADJ_ITERS_NOMINAL) if adj_iters is None else \
        np.maximum(np.asarray(adj_iters, np.float64), 1.0)
    return cells * (fi + ADJ_WEIGHT * nf * ai)


def split_by_cost(costs, size):
    """Per rank, the sorted solve indices of a longest-first greedy split of
    `costs` over `size` ranks (ties: the lower rank)."""
    costs = np.asarray(costs, np.float64)
    load = np.zeros(size)
    owner = np.empty(len(costs), np.int64)
    for s in np.argsort(-costs, kind="stable"):
        r = int(np.argmin(load))
        owner[s] = r
        load[r] += costs[s]
    return [np.flatnonzero(owner == r) for r in range(size)]


def shard_solves(pb, size, rank, by="cost", fwd_iters=None, adj_iters=None):
    """Solve indices of `rank`'s shard, in work-list order."""
    if by == "count":
        a, b = scatter_all_i(pb.nsolve, size, rank)
        return np.arange(a - 1, b)
    return split_by_cost(solve_costs(pb, fwd_iters, adj_iters), size)[rank]


def shard(pb, size, rank, by="cost", fwd_iters=None, adj_iters=None):
    """The rank's sub-problem: the same periods and path table, its solves
    only (global path indices kept, so tt_fwd lines up across ranks)."""
    solves = shard_solves(pb, size, rank, by, fwd_iters, adj_iters)
    sub = pb.subset(solves)
    idx = np.concatenate([np.arange(pb.rec_off[s], pb.rec_off[s] + pb.nrec[s]) for s in solves]) \
        if len(solves) else np.zeros(0, np.int64)
    sub.path = pb.path[idx].astype(np.int32)
    sub.n_paths = pb.npath
    return sub


def reduce_results(res, dist, device=None):
    """Sum-reduce one rank's result dict over the process group (all ranks
    receive the sums): adj_s, adj_density, tt_fwd and chi, packed into one
    buffer and reduced with one collective (on `device` when given)."""
    import torch
    keys = [k for k in ("adj_s", "adj_density", "tt_fwd") if res.get(k) is not None]
    parts = [np.ascontiguousarray(res[k], dtype=np.float64).ravel() for k in keys]
    flat = np.concatenate(parts + [np.array([float(res["chi"])])])
    t = torch.from_numpy(flat)
    if device is not None:
        t = t.to(device)
    dist.all_reduce(t)
    tot = t.cpu().numpy()
    out, o = dict(res), 0
    for k, a in zip(keys, parts):
        out[k] = tot[o:o + a.size].copy()
        o += a.size
    out["chi"] = float(tot[o])
    return out


def reduce_device(fields, dist):
    """The multi-GPU form of reduce_results: `fields` are device tensors (an
    engine's device_results()); they are copied into one device buffer,
    summed over the ranks with one collective, and returned as views of it
    (adj_s, adj_density, tt_fwd, chi; absent fields stay None)."""
    import torch
    keys = [k for k in ("adj_s", "adj_density", "tt_fwd", "chi") if fields.get(k) is not None]
    buf = torch.cat([fields[k].reshape(-1) for k in keys])
    dist.all_reduce(buf)
    out, o = {k: None for k in ("adj_s", "adj_density", "tt_fwd", "chi")}, 0
    for k in keys:
        n = fields[k].numel()
        out[k] = buf[o:o + n]
        o += n
    return out
