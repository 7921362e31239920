"""CUDA-graph replay of the gradient evaluation (GPU): a replayed evaluation
gives bitwise the results of the same evaluation enqueued launch by launch,
picks up a velocity update without a new capture, and a new load (another
shape) captures again."""
import numpy as np
import pytest

from surfatt_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _run(eng, mode, prec):
    eng.run(mode, prec)
    eng.sync()
    return eng.results()


def _same(x, y):
    return all(np.array_equal(x[k], y[k]) for k in ("adj_s", "adj_density", "tt_fwd")) and \
        x["chi"] == y["chi"]


@pytest.mark.parametrize("prec_name", ["PREC_FP64", "PREC_FP32"])
def test_graph_replay_equals_direct(sg, prec_name):
    prec = getattr(sg, prec_name)
    pb = W.flat_case(nx=70, ny=64, nsta=6, nperiod=2, mode=3, seed=21)
    eng = sg.Engine(0)
    eng.load(pb)
    eng.set_graphs(False)
    direct = _run(eng, 3, prec)
    eng.set_graphs(True)
    first = _run(eng, 3, prec)    # captures
    second = _run(eng, 3, prec)   # replays
    assert _same(direct, first) and _same(direct, second)
    # a velocity update is visible to the replayed graph
    v2 = pb.svel * (1.0 + 0.02 * np.sin(np.arange(pb.ncell) / 17.0))
    eng.update_velocity(v2)
    replay = _run(eng, 3, prec)
    eng.set_graphs(False)
    direct2 = _run(eng, 3, prec)
    assert _same(replay, direct2)
    assert not np.array_equal(replay["tt_fwd"], direct["tt_fwd"])
    eng.close()


def test_reload_recaptures(sg):
    a = W.flat_case(nx=64, ny=60, nsta=5, nperiod=2, mode=2, seed=22)
    b = W.flat_case(nx=90, ny=84, nsta=7, nperiod=3, mode=2, seed=23)
    eng = sg.Engine(0)
    outs = []
    for pb in (a, b, a):
        eng.load(pb)
        outs.append(_run(eng, 2, sg.PREC_FP64))
        outs.append(_run(eng, 2, sg.PREC_FP64))
    ref = sg.Engine(0)
    ref.set_graphs(False)
    for i, pb in enumerate((a, b, a)):
        ref.load(pb)
        r = _run(ref, 2, sg.PREC_FP64)
        assert _same(outs[2 * i], r) and _same(outs[2 * i + 1], r)
    assert len(outs[0]["tt_fwd"]) == a.npath and len(outs[2]["tt_fwd"]) == b.npath
    eng.close()
    ref.close()


def test_reload_same_shape_reuses_capture(sg):
    """A load of a problem with the same sizes keeps the captured graph (its
    sizes and buffers are unchanged); the replay computes the new problem."""
    a = W.flat_case(nx=72, ny=66, nsta=5, nperiod=2, mode=3, seed=24)
    b = W.flat_case(nx=72, ny=66, nsta=5, nperiod=2, mode=3, seed=25, vel=3.3)
    assert a.nsolve == b.nsolve and a.npath == b.npath
    eng = sg.Engine(0)
    eng.load(a)
    first = _run(eng, 3, sg.PREC_FP32)
    eng.load(b)
    replay = _run(eng, 3, sg.PREC_FP32)
    ref = sg.Engine(0)
    ref.set_graphs(False)
    ref.load(b)
    direct = _run(ref, 3, sg.PREC_FP32)
    assert _same(replay, direct)
    assert not np.array_equal(first["tt_fwd"], replay["tt_fwd"])
    eng.close()
    ref.close()
