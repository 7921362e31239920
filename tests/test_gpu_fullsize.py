"""The measured configurations themselves against the oracle (GPU only).

* Config 3 at full size: 80 stations x 16 periods = 1280 solves on 120 x
  120 grids, 3-D mode (two adjoints per solve), through the batched engine
  in plain FP64 and in the FP32-factored form, every period's travel times
  at the receivers, misfit and kernels (src/measadj.f90:62-104,
  src/acqui.f90:307-316), plus whole travel-time fields of a sample of
  solves against the oracle's FSM_UW_PS_lonlat_2d.
* Config 4 sampled: two sources x all 25 periods (grids 64^2 ... 384^2:
  every warp-team class of the FP32 row kernel), FP64 and FP32.
* A serving request on the curved-surface metric of config 5 (a gradient
  evaluation of a 128^2 grid through the serving loop).

Tolerances: plain FP64 travel times and misfit 1e-6 (pointwise / relative),
kernels 1e-5 (norm-wise per period); FP32-factored 1e-5 / 1e-3.
"""
import os

import numpy as np
import pytest

from conftest import rel_max, rel_pointwise
from surfatt_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TT64, KER64 = 1e-6, 1e-5
TT32, KER32 = 1e-5, 1e-3
NTHR = os.cpu_count() or 1


def _per_period(got, ref, pb, tt_tol, ker_tol, chi_tol):
    """Every period: receiver times, the period's misfit, adj_s, adj_density."""
    pid = np.asarray(pb.pidx)
    for p in range(pb.nperiod):
        sol = np.flatnonzero(pid == p)
        if len(sol) == 0:
            continue
        ridx = np.concatenate([np.arange(pb.rec_off[s], pb.rec_off[s] + pb.nrec[s]) for s in sol])
        paths = np.asarray(pb.path)[ridx]
        assert rel_pointwise(got["tt_fwd"][paths], ref["tt_fwd"][paths]) <= tt_tol, p
        w, tt = np.asarray(pb.weight)[ridx], np.asarray(pb.tt)[ridx]
        cg = 0.5 * np.sum(w * (got["tt_fwd"][paths] - tt) ** 2)
        cr = 0.5 * np.sum(w * (ref["tt_fwd"][paths] - tt) ** 2)
        assert abs(cg - cr) <= chi_tol * abs(cr), p
        g0, n = int(pb.goff[p]), int(pb.nx[p] * pb.ny[p])
        for key in ("adj_s", "adj_density"):
            assert rel_max(got[key][g0:g0 + n], ref[key][g0:g0 + n]) <= ker_tol, (key, p)
    assert abs(got["chi"] - ref["chi"]) <= chi_tol * abs(ref["chi"])


def _fields_vs_oracle(oracle, pb, fields, solves, tol):
    for s in solves:
        p = int(pb.pidx[s])
        xx, yy = pb.grid(p)
        m11, m12, m22 = (pb.field(k, p) for k in ("m11", "m12", "m22"))
        Tr, st, _ = oracle.fsm_uw_ps_lonlat_2d(xx, yy, m11, m22, -m12, 1.0 / pb.field("svel", p),
                                               float(pb.srcx[s]), float(pb.srcy[s]))
        assert st == 0
        assert rel_pointwise(fields[s], Tr) <= tol, s


@pytest.fixture(scope="module")
def config3(oracle):
    pb = W.config2()
    assert pb.nsolve == 1280 and set(pb.nx) == {120} and pb.mode == 3
    return pb, oracle.gradient_eval(pb, mode=3, nthreads=NTHR)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_config3_full_size(sg, oracle, config3, prec):
    pb, ref = config3
    eng = sg.Engine(0)
    eng.load(pb)
    eng.set_keep_fields(True)
    p = sg.PREC_FP64 if prec == "fp64" else sg.PREC_FP32
    got = eng.evaluate(mode=3, precision=p)
    assert int(np.max(got["status"])) == 0
    tt, ker = (TT64, KER64) if prec == "fp64" else (TT32, KER32)
    _per_period(got, ref, pb, tt, ker, tt)
    if prec == "fp64":
        assert np.array_equal(got["fwd_iters"], ref["fwd_iters"])
    # whole travel-time fields: 24 solves spread over the periods and stations
    sample = np.linspace(0, pb.nsolve - 1, 24).astype(int)
    _fields_vs_oracle(oracle, pb, eng.fields(), sample, tt)
    eng.close()


def _config4_sample():
    full = W.config4()
    nsrc = 120
    sel = np.array([p * nsrc + s for p in range(full.nperiod) for s in (0, 57)])
    return full.subset(sel)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_config4_sampled(sg, oracle, prec):
    pb = _config4_sample()
    sides = sorted({int(n) for n in pb.ny})
    assert sides[0] == 64 and sides[-1] == 384
    # every team class of the row kernel: 1 warp (<= 128 rows), 2, 3
    assert {1 if n <= 128 else (n + 127) // 128 for n in sides} == {1, 2, 3}
    ref = oracle.gradient_eval(pb, mode=3, nthreads=NTHR)
    eng = sg.Engine(0)
    eng.load(pb)
    eng.set_keep_fields(True)
    p = sg.PREC_FP64 if prec == "fp64" else sg.PREC_FP32
    got = eng.evaluate(mode=3, precision=p)
    assert int(np.max(got["status"])) == 0
    tt, ker = (TT64, KER64) if prec == "fp64" else (TT32, KER32)
    _per_period(got, ref, pb, tt, ker, tt)
    # whole fields of the largest and the smallest grids
    big = [s for s in range(pb.nsolve) if int(pb.ny[pb.pidx[s]]) in (sides[0], sides[-1])]
    _fields_vs_oracle(oracle, pb, eng.fields(), big, tt)
    eng.close()


def test_config4_every_fp32_variant_same_bits(sg):
    """Config 4's uneven grids (six sources x all 25 periods, 64^2 ... 384^2)
    through every variant of the FP32 row kernel -- teams or strips, work
    items or whole solves, operands a step ahead or at the visit: the same
    bits everywhere (travel times, kernels, misfit, iteration counts)."""
    pb = W.config4(nsrc=6)
    eng = sg.Engine(0)
    eng.load(pb)
    outs = {}
    for v in range(6):
        eng.set_kernel(sg.PREC_FP32, kind=2, variant=v)
        eng.run(3, sg.PREC_FP32)
        assert eng.sync() == sg.OK
        outs[v] = eng.results()
    eng.close()
    base = outs[0]
    assert int(np.max(base["status"])) == 0
    for v in range(1, 6):
        for k in ("tt_fwd", "adj_s", "adj_density", "fwd_iters", "adj_iters", "status"):
            assert np.array_equal(outs[v][k], base[k]), (v, k)
        assert outs[v]["chi"] == base["chi"], v


def test_serving_request_on_curved_surface(sg, oracle):
    """One gradient request (3-D mode) over the surface metric of the
    config-5 island (resampled to 128^2) through the serving loop, FP64 and
    FP32, against the oracle's evaluation of the same work list."""
    from surfatt_gb300 import serving as S
    cat = S.Catalog(sides=(128,), nperiod=4, nsta=30)
    pb = cat.worklist(128, np.arange(0, 30, 3), np.array([0, 3]), 3, seed=9)
    m = pb.field("m12", 0)
    assert np.max(np.abs(m)) > 1e-3  # a curved surface: the metric is not flat
    ref = oracle.gradient_eval(pb, mode=3, nthreads=NTHR)
    srv = sg.Server(0, hbm_budget_bytes=2 << 30, max_inflight=2)
    wl = srv.add_worklist(srv.add_model(cat.models[128]), pb)
    for prec, tt, ker in ((sg.PREC_FP64, TT64, KER64), (sg.PREC_FP32, TT32, KER32)):
        st, got, _ = srv.wait(srv.submit(wl, None, 3, prec))
        assert st == sg.OK
        _per_period(got, ref, pb, tt, ker, tt)
    srv.close()


def test_bounded_item_wait_times_out(sg, oracle):
    """The FP32 row kernel's wait for a solve's previous work item is
    bounded: with the test hook, the first item of one solve is never marked
    done, its next item gives up after a short poll limit and reports
    SURFATT_TIMEOUT, the solve contributes nothing, every other solve
    matches the oracle, and the next run (hook off) is clean."""
    pb = W.config2(nsta=12, nperiod=3)
    held = 7
    eng = sg.Engine(0)
    eng.load(pb)
    eng.set_kernel(sg.PREC_FP32, 2, 0)  # row kernel, register prefetch, work items
    clean = eng.evaluate(mode=3, precision=sg.PREC_FP32)
    assert int(np.max(clean["status"])) == 0
    eng.test_hold(held, 2000)
    got = eng.evaluate(mode=3, precision=sg.PREC_FP32)
    assert got["status"][held] == sg.TIMEOUT
    assert got["fwd_iters"][held] == 0
    others = np.delete(np.arange(pb.nsolve), held)
    assert np.all(got["status"][others] == sg.OK)
    # everything else equals the oracle on the work list without that solve
    sub = pb.subset(others)
    ref = oracle.gradient_eval(sub, mode=3, nthreads=NTHR)
    r0, n = int(pb.rec_off[held]), int(pb.nrec[held])
    assert np.all(got["tt_fwd"][pb.path[r0:r0 + n]] == 0.0)
    # the subset's paths are the remaining solves' receivers in order
    ridx = np.concatenate([np.arange(pb.rec_off[s], pb.rec_off[s] + pb.nrec[s]) for s in others])
    assert rel_pointwise(got["tt_fwd"][pb.path[ridx]], ref["tt_fwd"][sub.path]) <= TT32
    for key in ("adj_s", "adj_density"):
        assert rel_max(got[key], ref[key]) <= KER32
    assert abs(got["chi"] - ref["chi"]) <= TT32 * ref["chi"]
    # hook off: the next run gives the clean run's bits again
    eng.test_hold(-1, 0)
    again = eng.evaluate(mode=3, precision=sg.PREC_FP32)
    for key in ("adj_s", "adj_density", "tt_fwd"):
        assert np.array_equal(again[key], clean[key])
    assert np.array_equal(again["status"], clean["status"])
    eng.close()
