"""Kernel smoothing (gaussian_smooth_geo_2, src/shared/utils.f90:1194-1225) on
the GPU vs the oracle (GPU only).

The GPU form evaluates each great-circle weight once per (row, window row,
column offset) instead of once per tap, uses fma for the weighted sum and
prefix sums for the weight sum, so it differs from the reference's
evaluation order by rounding only.  Tolerance: norm-wise relative error
<= 1e-12 per field (the path's kernel bar is 1e-5).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_max
from surfatt_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SMOOTH_TOL = 1e-12
KER_TOL = 1e-5


def _field(nx, ny, seed):
    rng = np.random.default_rng(seed)
    # smooth large-scale part plus node-to-node noise, both signs (like adj_s)
    x = np.linspace(0, 3, nx)[:, None]
    y = np.linspace(0, 2, ny)[None, :]
    return np.sin(2.1 * x) * np.cos(1.7 * y) + 0.3 * rng.standard_normal((nx, ny))


@pytest.mark.parametrize("nx,ny,x0,y0,d,sigma", [
    (81, 81, 100.0, 22.0, 0.05, 0.2),     # config-1 grid, the example's sigma_2d
    (37, 23, 100.0, 22.0, 0.05, 0.12),    # non-square, odd sizes
    (120, 96, 96.0, -35.0, 0.05, 0.3),    # southern hemisphere, 3 sigma / dx = 18
    (150, 64, 100.0, 30.0, 0.02, 0.05),   # fine grid, wide window in rows
    (17, 13, 100.0, 22.0, 0.05, 1.0),     # window wider than the grid (clamped)
    (29, 31, 100.0, 22.0, 0.05, 0.01),    # 3 sigma < dx: one-column window
    (200, 40, 100.0, 60.0, 0.05, 0.2),    # high latitude: row window grows with 1/cos
])
def test_dropin_matches_oracle(sg, oracle, nx, ny, x0, y0, d, sigma):
    lons, lats = W.arange_grid(x0, nx, d), W.arange_grid(y0, ny, d)
    data = _field(nx, ny, nx * 1000 + ny)
    got = sg.gaussian_smooth_geo_2(data, lons, lats, sigma)
    ref = oracle.gaussian_smooth_geo_2(data, lons, lats, sigma)
    assert got.shape == ref.shape
    assert rel_max(got, ref) <= SMOOTH_TOL


def test_dropin_constant_and_spike(sg, oracle):
    lons, lats = W.arange_grid(100.0, 41, 0.05), W.arange_grid(22.0, 33, 0.05)
    c = sg.gaussian_smooth_geo_2(np.full((41, 33), -1.25), lons, lats, 0.15)
    assert np.max(np.abs(c + 1.25)) <= 1e-13
    spike = np.zeros((41, 33))
    spike[20, 16] = 1.0
    got = sg.gaussian_smooth_geo_2(spike, lons, lats, 0.1)
    ref = oracle.gaussian_smooth_geo_2(spike, lons, lats, 0.1)
    # identical support: the window truncations agree exactly
    assert np.array_equal(got != 0, ref != 0)
    assert rel_max(got, ref) <= SMOOTH_TOL


def _f(pb, a, p):
    """(nx, ny) view of period p of a packed per-cell array."""
    nx, ny, g = int(pb.nx[p]), int(pb.ny[p]), int(pb.goff[p])
    return a[g:g + nx * ny].reshape((nx, ny), order="F")


def _grid(pb, p):
    return (pb.xgrid[pb.xoff[p]:pb.xoff[p] + pb.nx[p]],
            pb.ygrid[pb.yoff[p]:pb.yoff[p] + pb.ny[p]])


@pytest.mark.parametrize("mode", [2, 3])
def test_engine_smooth_matches_oracle(sg, oracle, mode):
    """ker_s of every period (uneven grids) from the engine's resident adj_s
    equals the oracle's smoothing of the same adj_s."""
    pb = W.config4(nsrc=6, nperiod=3, nmax=72, nmin=40, span_deg=2.0, seed=31, mode=mode)
    eng = sg.Engine(0)
    eng.load(pb)
    eng.run(mode, sg.PREC_FP64)
    eng.sync()
    adj = eng.results()["adj_s"]
    ker = eng.smooth(0.15)
    for p in range(pb.nperiod):
        lons, lats = _grid(pb, p)
        ref = oracle.gaussian_smooth_geo_2(_f(pb, adj, p), lons, lats, 0.15)
        assert rel_max(_f(pb, ker, p), ref) <= SMOOTH_TOL
    # device-only form, a second sigma (new window plan and table), then the
    # same sigma again (table kept: apply only), then the first sigma again
    assert eng.smooth(0.25, host=False) is None
    assert eng.sync() == 0
    ms, taps, n = eng.smooth_timing()
    assert ms > 0 and taps > 0 and n == 2
    k25 = eng.smooth(0.25)
    assert eng.smooth_timing()[2] == 1
    for p in range(pb.nperiod):
        lons, lats = _grid(pb, p)
        ref = oracle.gaussian_smooth_geo_2(_f(pb, adj, p), lons, lats, 0.25)
        assert rel_max(_f(pb, k25, p), ref) <= SMOOTH_TOL
    again = eng.smooth(0.15)
    assert np.array_equal(again, ker)
    # a new adj_s (velocity update) smoothed with the kept table
    eng.update_velocity(pb.svel * 1.01)
    eng.run(mode, sg.PREC_FP64)
    eng.sync()
    adj2 = eng.results()["adj_s"]
    ker2 = eng.smooth(0.15)
    assert eng.smooth_timing()[2] == 1
    for p in range(pb.nperiod):
        lons, lats = _grid(pb, p)
        ref = oracle.gaussian_smooth_geo_2(_f(pb, adj2, p), lons, lats, 0.15)
        assert rel_max(_f(pb, ker2, p), ref) <= SMOOTH_TOL
    eng.close()


def test_dropin_table_reuse(sg, oracle):
    """Consecutive drop-in calls on one grid with one sigma reuse the weight
    table; a change of data, sigma or grid values gives the oracle's answer."""
    lons, lats = W.arange_grid(100.0, 50, 0.05), W.arange_grid(22.0, 44, 0.05)
    cases = [(_field(50, 44, 1), lons, lats, 0.2), (_field(50, 44, 2), lons, lats, 0.2),
             (_field(50, 44, 3), lons, lats, 0.15),
             (_field(50, 44, 4), lons + 0.5, lats, 0.15),
             (_field(50, 44, 5), lons + 0.5, lats - 1.0, 0.15)]
    for data, lo, la, sig in cases:
        got = sg.gaussian_smooth_geo_2(data, lo, la, sig)
        ref = oracle.gaussian_smooth_geo_2(data, lo, la, sig)
        assert rel_max(got, ref) <= SMOOTH_TOL


def test_engine_smooth_requires_adjoint_run(sg):
    pb = W.flat_case(nx=40, ny=36, nsta=4, nperiod=1, mode=0, seed=32)
    eng = sg.Engine(0)
    eng.load(pb)
    with pytest.raises(sg.SurfattError):
        eng.smooth(0.1)
    eng.run(0, sg.PREC_FP64)
    eng.sync()
    with pytest.raises(sg.SurfattError):
        eng.smooth(0.1)   # forward-only run: no adj_s
    eng.close()


def test_tomo2d_gradient_then_smoothing_vs_oracle(sg, oracle):
    """The tomo2d optimize input end to end: FP64 gradient evaluation then
    smoothing on the GPU vs the oracle's evaluation then its smoothing
    (kernel bar 1e-5 per period)."""
    obs = W.read_src_rec_tt(os.path.join(GOLDEN, "config1_src_rec.csv"))
    pb = W.config1(observed_tt=obs)
    eng = sg.Engine(0)
    eng.load(pb)
    eng.run(2, sg.PREC_FP64)
    eng.sync()
    ker = eng.smooth(0.2)
    ref = oracle.gradient_eval(pb, mode=2, nthreads=8)
    lons, lats = _grid(pb, 0)
    ker_ref = oracle.gaussian_smooth_geo_2(_f(pb, ref["adj_s"], 0), lons, lats, 0.2)
    assert rel_max(_f(pb, ker, 0), ker_ref) <= KER_TOL
    eng.close()
