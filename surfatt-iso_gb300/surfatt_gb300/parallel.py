"""Work-list sharding over ranks (one GPU per rank).

The reference splits its (period, source) work list into contiguous blocks,
one per MPI rank (scatter_all_i, src/shared/parallel.f90:1877-1903,
src/src_rec.f90:368), and sums the per-period kernels, the misfit and the
synthetic-time table to rank 0 (MPI_Reduce, src/acqui.f90:152-160,
src/tomo2d.f90:196-200).  The same split and the same sums are used here:
each rank evaluates its block on its own GPU, then one sum-reduction of
(adj_s, adj_density, chi, tt_fwd) -- the path's only exchange step.
"""
import numpy as np


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


def shard(pb, size, rank):
    """The rank's sub-problem (same periods and path table, its solves only)."""
    a, b = scatter_all_i(pb.nsolve, size, rank)
    solves = np.arange(a - 1, b)
    sub = pb.subset(solves)
    # keep the global path indices so tt_fwd lines up across ranks
    idx = np.concatenate([np.arange(pb.rec_off[s], pb.rec_off[s] + pb.nrec[s]) for s in solves]) \
        if len(solves) else np.zeros(0, np.int64)
    sub.path = pb.path[idx].astype(np.int32)
    sub.n_paths = pb.npath
    return sub


def reduce_results(res, dist, device=None):
    """Sum-reduce one rank's result dict over the process group (all ranks
    receive the sums): adj_s, adj_density, tt_fwd and chi."""
    import torch
    out = dict(res)
    for key in ("adj_s", "adj_density", "tt_fwd"):
        if key in res:
            t = torch.from_numpy(np.ascontiguousarray(res[key], dtype=np.float64))
            if device is not None:
                t = t.to(device)
            dist.all_reduce(t)
            out[key] = t.cpu().numpy()
    c = torch.tensor([float(res["chi"])], dtype=torch.float64)
    if device is not None:
        c = c.to(device)
    dist.all_reduce(c)
    out["chi"] = float(c.cpu()[0])
    return out
