"""Serving loop (GPU): requests admitted by an HBM budget run concurrently,
and each result is the same alone and in the mix (bitwise: per-solve work is
independent of scheduling and the per-period sums are ordered)."""
import numpy as np
import pytest

from surfatt_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _model_and_lists():
    a = W.flat_case(nx=64, ny=60, nsta=6, nperiod=3, mode=3, seed=11)
    b = W.flat_case(nx=96, ny=90, nsta=5, nperiod=2, mode=2, seed=12)
    return a, b


def _same(x, y):
    return (np.array_equal(x["adj_s"], y["adj_s"]) and
            np.array_equal(x["adj_density"], y["adj_density"]) and
            np.array_equal(x["tt_fwd"], y["tt_fwd"]) and x["chi"] == y["chi"])


def test_alone_equals_in_the_mix(sg):
    a, b = _model_and_lists()
    srv = sg.Server(0, hbm_budget_bytes=2 << 30, max_inflight=4)
    ma, mb = srv.add_model(a), srv.add_model(b)
    wa, wb = srv.add_worklist(ma, a), srv.add_worklist(mb, b)
    trial = a.svel * 1.01  # a line-search trial model
    reqs = [(wa, None, 3, sg.PREC_FP64), (wb, None, 2, sg.PREC_FP32),
            (wa, trial, 3, sg.PREC_FP32), (wb, None, 0, sg.PREC_FP64),
            (wa, None, 2, sg.PREC_FP32), (wb, b.svel * 0.99, 2, sg.PREC_FP64)]
    alone = []
    for wl, v, mode, prec in reqs:
        st, res, _ = srv.wait(srv.submit(wl, v, mode, prec))
        assert st == sg.OK
        alone.append(res)
    tickets = [srv.submit(wl, v, mode, prec) for wl, v, mode, prec in reqs]
    mixed = [srv.wait(t) for t in tickets]
    for (st, res, lat), ref in zip(mixed, alone):
        assert st == sg.OK
        assert lat > 0
        assert _same(res, ref)
    stats = srv.stats()
    assert stats["completed"] == 2 * len(reqs)
    assert stats["inflight_peak"] >= 2
    srv.close()


def test_team_classes_alone_equals_in_the_mix(sg):
    """A request whose grids need warp teams of three sizes (48 to 304 rows:
    one launch per team class on the request's side streams) gives the same
    bits alone, in the mix with other requests, and through the engine."""
    c = W.config4(nsrc=4, nperiod=5, nmax=300, nmin=48, span_deg=2.0, seed=43)
    assert {1 if n <= 128 else (int(n) + 127) // 128 for n in c.ny} == {1, 2, 3}
    a, _ = _model_and_lists()
    srv = sg.Server(0, hbm_budget_bytes=4 << 30, max_inflight=4)
    wc = srv.add_worklist(srv.add_model(c), c)
    wa = srv.add_worklist(srv.add_model(a), a)
    reqs = [(wc, None, 3, sg.PREC_FP32), (wa, None, 3, sg.PREC_FP32),
            (wc, c.svel * 1.01, 2, sg.PREC_FP32), (wc, None, 3, sg.PREC_FP64)]
    alone = []
    for wl, v, mode, prec in reqs:
        st, res, _ = srv.wait(srv.submit(wl, v, mode, prec))
        assert st == sg.OK
        alone.append(res)
    tickets = [srv.submit(wl, v, mode, prec) for wl, v, mode, prec in reqs]
    for t, ref in zip(tickets, alone):
        st, res, _ = srv.wait(t)
        assert st == sg.OK
        assert _same(res, ref)
    srv.close()
    eng = sg.Engine(0)
    ref = eng.evaluate(c, mode=3, precision=sg.PREC_FP32)
    eng.close()
    assert np.array_equal(alone[0]["adj_s"], ref["adj_s"])
    assert np.array_equal(alone[0]["tt_fwd"], ref["tt_fwd"])


def test_server_matches_engine(sg):
    a, _ = _model_and_lists()
    srv = sg.Server(0, hbm_budget_bytes=1 << 30, max_inflight=2)
    wa = srv.add_worklist(srv.add_model(a), a)
    st, res, _ = srv.wait(srv.submit(wa, None, 3, sg.PREC_FP64))
    assert st == sg.OK
    eng = sg.Engine(0)
    ref = eng.evaluate(a, mode=3)
    assert np.array_equal(res["adj_s"], ref["adj_s"])
    assert np.array_equal(res["tt_fwd"], ref["tt_fwd"])
    eng.close()
    srv.close()


def test_request_larger_than_budget_fails_cleanly(sg):
    a, _ = _model_and_lists()
    srv = sg.Server(0, hbm_budget_bytes=8 << 20, max_inflight=2)
    wa = srv.add_worklist(srv.add_model(a), a)
    st, _, _ = srv.wait(srv.submit(wa, None, 3, sg.PREC_FP64), timeout_s=60)
    assert st == sg.OOM
    srv.close()
