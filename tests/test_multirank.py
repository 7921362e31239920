"""Work-list sharding over 2 ranks (gloo, CPU): each rank evaluates its
contiguous block (scatter_all_i) and the per-period kernels, misfit and
synthetic-time table are sum-reduced -- the reference's MPI_Reduce step.
The sum of the shards must equal the single-process evaluation."""
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


def _worker(rank, world, port, q):
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "surfatt-iso_gb300"))
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import torch.distributed as dist
    import oracle as O
    from surfatt_gb300 import parallel as par
    from surfatt_gb300 import workloads as W
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pb = W.flat_case(nx=28, ny=26, nsta=5, nperiod=2, mode=3)
    sub = par.shard(pb, world, rank)
    r = O.gradient_eval(sub, mode=3, nthreads=1)
    tot = par.reduce_results(r, dist)
    if rank == 0:
        q.put({k: tot[k] for k in ("adj_s", "adj_density", "tt_fwd", "chi")})
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shards_sum_to_full(oracle):
    import multiprocessing as mp
    from surfatt_gb300 import workloads as W
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    pb = W.flat_case(nx=28, ny=26, nsta=5, nperiod=2, mode=3)
    full = oracle.gradient_eval(pb, mode=3, nthreads=1)
    assert np.array_equal(res["tt_fwd"], full["tt_fwd"])
    assert np.max(np.abs(res["adj_s"] - full["adj_s"])) <= 1e-12 * np.max(np.abs(full["adj_s"]))
    assert np.max(np.abs(res["adj_density"] - full["adj_density"])) <= \
        1e-12 * np.max(np.abs(full["adj_density"]))
    assert abs(res["chi"] - full["chi"]) <= 1e-12 * full["chi"]
