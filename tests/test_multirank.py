"""Work-list sharding over 2 ranks (gloo, CPU): each rank evaluates its shard
and the per-period kernels, misfit and synthetic-time table are sum-reduced
-- the reference's MPI_Reduce step (src/acqui.f90:152-160, 205-206).  The
sum of the shards must equal the single-process evaluation, for the
reference's count split (scatter_all_i) on a uniform work list and for the
cost split on a work list whose grids differ between periods."""
import os
import socket
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _uniform():
    from surfatt_gb300 import workloads as W
    return W.flat_case(nx=28, ny=26, nsta=5, nperiod=2, mode=3)


def _uneven():
    # six periods whose grids go from 40^2 down to 16^2 over the same box,
    # period-major work list (all large grids first), 8 sources
    from surfatt_gb300 import workloads as W
    return W.config4(nsrc=8, nperiod=6, nmax=40, nmin=16, span_deg=2.0)


def _worker(rank, world, port, q, case, by):
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "surfatt-iso_gb300"))
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import torch.distributed as dist
    import oracle as O
    from surfatt_gb300 import parallel as par
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pb = _uniform() if case == "uniform" else _uneven()
    sub = par.shard(pb, world, rank, by=by)
    r = O.gradient_eval(sub, mode=3, nthreads=1)
    tot = par.reduce_results(r, dist)
    if rank == 0:
        q.put({k: tot[k] for k in ("adj_s", "adj_density", "tt_fwd", "chi")})
    dist.barrier()
    dist.destroy_process_group()


def _run(case, by):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q, case, by)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    return res


def _check_sum(res, full):
    assert np.array_equal(res["tt_fwd"], full["tt_fwd"])
    for k in ("adj_s", "adj_density"):
        assert np.max(np.abs(res[k] - full[k])) <= 1e-12 * np.max(np.abs(full[k]))
    assert abs(res["chi"] - full["chi"]) <= 1e-12 * full["chi"]


def test_two_rank_shards_sum_to_full(oracle):
    res = _run("uniform", "count")
    _check_sum(res, oracle.gradient_eval(_uniform(), mode=3, nthreads=1))


def test_two_rank_cost_split_uneven_grids(oracle):
    from surfatt_gb300 import parallel as par
    pb = _uneven()
    assert len(set(int(n) for n in pb.nx)) >= 4  # grids differ between periods
    costs = par.solve_costs(pb)
    shards = [par.shard_solves(pb, 2, r) for r in range(2)]
    # every solve in exactly one shard, each shard in work-list order
    assert np.array_equal(np.sort(np.concatenate(shards)), np.arange(pb.nsolve))
    assert all(np.all(np.diff(s) > 0) for s in shards)
    load = [costs[s].sum() for s in shards]
    assert max(load) <= 1.10 * min(load)
    # the count split of the same work list is far from balanced
    cnt = [costs[par.shard_solves(pb, 2, r, by="count")].sum() for r in range(2)]
    assert max(cnt) > 1.5 * min(cnt)
    res = _run("uneven", "cost")
    _check_sum(res, oracle.gradient_eval(pb, mode=3, nthreads=1))


def test_cost_model_uses_previous_iterations():
    from surfatt_gb300 import parallel as par
    pb = _uneven()
    base = par.solve_costs(pb)
    fit = np.full(pb.nsolve, 5.0)
    fit[0] = 50.0  # a solve that took ten times the iterations last time
    c = par.solve_costs(pb, fwd_iters=fit, adj_iters=np.full(pb.nsolve, 3.0))
    assert c[0] > 5 * base[0] and np.allclose(c[1:], base[1:])
    # four ranks: every solve placed once, loads within one largest solve
    sh = par.split_by_cost(c, 4)
    assert sorted(np.concatenate(sh).tolist()) == list(range(pb.nsolve))
    load = np.array([c[s].sum() for s in sh])
    assert load.max() - load.min() <= c.max()
