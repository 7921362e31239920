"""Pins of the CPU oracle (no GPU needed).

The reference ships no golden vectors for this path and cannot be built here,
so the oracle is pinned by: the committed fixtures (detect any change), an
analytic homogeneous-medium answer, reciprocity, a finite-difference check of
the adjoint kernel, and invariance to the thread split.
"""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_max, rel_pointwise
from surfatt_gb300 import workloads as W


def test_small_case_fixtures(oracle):
    g = np.load(os.path.join(GOLDEN, "small_cases.npz"))
    xx, yy, fun = g["fw_xx"], g["fw_yy"], g["fw_fun"]
    one = np.ones_like(fun)
    T, st, it = oracle.fsm_uw_ps_lonlat_2d(xx, yy, one, one, 0 * one, fun, *g["fw_src"])
    assert st == 0 and it == g["fw_iters"][0]
    assert rel_pointwise(T, g["fw_T"]) <= 1e-12
    Ta, st, it = oracle.fsm_o1_jse_lonlat_2d(xx, yy, one, one, 0 * one, g["fw_T"], g["adj_xr"],
                                            g["adj_yr"], g["adj_s"])
    assert st == 0 and it == g["adj_iters"][0]
    assert rel_max(Ta, g["adj_Ta"]) <= 1e-12
    assert np.array_equal(oracle.mask(xx, yy, g["adj_Ta"], *g["fw_src"]), g["mask_T"])
    v = [oracle.interp2(xx, yy, g["fw_T"], x, y) for x, y in zip(g["adj_xr"], g["adj_yr"])]
    assert np.allclose(v, g["interp"], rtol=1e-14, atol=0)
    pb = W.flat_case(nx=27, ny=25, nsta=4, nperiod=2, mode=3)
    r = oracle.gradient_eval(pb, mode=3, nthreads=1)
    assert rel_max(r["adj_s"], g["ge_adj_s"]) <= 1e-12
    assert rel_max(r["adj_density"], g["ge_adj_density"]) <= 1e-12
    assert abs(r["chi"] - g["ge_chi"][0]) <= 1e-12 * abs(g["ge_chi"][0])
    assert np.array_equal(r["fwd_iters"], g["ge_fwd_iters"])


def test_config1_fixture(oracle):
    """The committed observed times of config 1 are the oracle's forward times
    on the checkerboard model (written with F0.6)."""
    tt = W.read_src_rec_tt(os.path.join(GOLDEN, "config1_src_rec.csv"))
    r = oracle.gradient_eval(W.config1_true_model(), mode=0, nthreads=4)
    assert r["rc"] == 0
    assert np.max(np.abs(r["tt_fwd"] - tt)) <= 5.1e-7


def test_homogeneous_known_answer(oracle):
    """Flat metric and constant velocity: tau == 1 is a fixed point, so T is
    the great-circle distance over v.  The reference interpolates the source
    slowness with REAL(4) weights, which bounds the agreement at ~1e-7."""
    nx, ny, v = 41, 37, 3.0
    xx, yy = W.arange_grid(100.0, nx, 0.05), W.arange_grid(22.0, ny, 0.05)
    one = np.ones((nx, ny))
    x0, y0 = 100.93, 22.81
    T, st, it = oracle.fsm_uw_ps_lonlat_2d(xx, yy, one, one, 0 * one, one / v, x0, y0)
    assert st == 0
    pi = float(np.float32(math.pi))
    X, Y = np.meshgrid(xx / 180 * pi, yy / 180 * pi, indexing="ij")
    la0, lo0 = y0 / 180 * pi, x0 / 180 * pi
    c = np.sin(Y) * np.sin(la0) + np.cos(Y) * np.cos(la0) * np.cos(X - lo0)
    ref = np.arccos(np.clip(c, -1, 1)) * 6371.0 / v
    assert rel_pointwise(T, ref) <= 3e-7


def test_reciprocity(oracle):
    """T_A(B) ~ T_B(A) within the first-order discretisation error."""
    nx, ny = 61, 55
    xx, yy = W.arange_grid(100.0, nx, 0.05), W.arange_grid(22.0, ny, 0.05)
    one = np.ones((nx, ny))
    fun = 1.0 / (3.0 * W.checkerboard_2d(nx, ny, 2, 3, 0.06))
    A, B = (100.52, 22.61), (102.41, 24.33)
    TA, _, _ = oracle.fsm_uw_ps_lonlat_2d(xx, yy, one, one, 0 * one, fun, *A)
    TB, _, _ = oracle.fsm_uw_ps_lonlat_2d(xx, yy, one, one, 0 * one, fun, *B)
    ab = oracle.interp2(xx, yy, TA, *B)
    ba = oracle.interp2(xx, yy, TB, *A)
    assert abs(ab - ba) / ab < 5e-3


def test_adjoint_kernel_finite_difference(oracle):
    """The 2-D kernel is the gradient of chi w.r.t. ln(velocity): for a smooth
    relative perturbation dm, chi(v*exp(h*dm)) - chi(v*exp(-h*dm)) over 2h
    matches -sum(K*dm)*dA (dA the cell area on the sphere, km^2) to the
    first-order discretisation error."""
    pb = W.flat_case(nx=45, ny=41, nsta=5, nperiod=1, mode=2, pert=0.0)
    xx, yy = pb.grid(0)
    r = oracle.gradient_eval(pb, mode=2, nthreads=4)
    K = r["adj_s"].reshape((45, 41), order="F")
    X, Y = np.meshgrid(np.arange(45), np.arange(41), indexing="ij")
    dm = 0.05 * np.sin(2 * np.pi * X / 44) * np.cos(np.pi * Y / 40)
    h = 1e-3
    base = pb.svel.reshape((45, 41), order="F").copy()
    chis = []
    for sgn in (1, -1):
        pb.svel = (base * np.exp(sgn * h * dm)).ravel(order="F")
        chis.append(oracle.gradient_eval(pb, mode=0, nthreads=4)["chi"])
    fd = (chis[0] - chis[1]) / (2 * h)
    d = math.radians(0.05) * 6371.0
    dA = d * d * np.cos(np.radians(yy))[None, :]
    pred = -np.sum(K * dm * dA)
    assert abs(fd - pred) <= 0.05 * abs(fd)


def test_thread_split_invariance(oracle):
    pb = W.flat_case(nx=30, ny=28, nsta=5, nperiod=2, mode=3)
    r1 = oracle.gradient_eval(pb, mode=3, nthreads=1)
    r4 = oracle.gradient_eval(pb, mode=3, nthreads=4)
    assert np.array_equal(r1["tt_fwd"], r4["tt_fwd"])
    assert rel_max(r4["adj_s"], r1["adj_s"]) <= 1e-13
    assert abs(r4["chi"] - r1["chi"]) <= 1e-13 * r1["chi"]


@pytest.mark.parametrize("count,size", [(10, 3), (2, 5), (7, 7), (0, 2), (100, 16)])
def test_scatter_all_i(oracle, count, size):
    """Contiguous block split of src/shared/parallel.f90:1877-1903."""
    from surfatt_gb300 import parallel as par
    seen = []
    for rank in range(size):
        a, b = oracle.scatter_all_i(count, size, rank)
        assert par.scatter_all_i(count, size, rank) == (a, b)
        seen += list(range(a, b + 1))
    assert seen == list(range(1, count + 1))


def test_interp2_semantics(oracle):
    """interp2_0_dp: node queries return the node value; outside raises."""
    xx, yy = W.arange_grid(0.0, 5, 1.0), W.arange_grid(0.0, 4, 1.0)
    v = np.arange(20, dtype=float).reshape((5, 4), order="F")
    assert oracle.interp2(xx, yy, v, 2.0, 1.0) == v[2, 1]
    assert abs(oracle.interp2(xx, yy, v, 2.5, 1.5) - 0.25 * (v[2, 1] + v[3, 1] + v[2, 2] + v[3, 2])) < 1e-14
    with pytest.raises(ValueError):
        oracle.interp2(xx, yy, v, 4.0, 1.0)
    with pytest.raises(ValueError):
        oracle.interp2(xx, yy, v, -0.5, 1.0)


def test_source_on_boundary(oracle):
    xx, yy = W.arange_grid(100.0, 20, 0.05), W.arange_grid(22.0, 20, 0.05)
    one = np.ones((20, 20))
    _, st, _ = oracle.fsm_uw_ps_lonlat_2d(xx, yy, one, one, 0 * one, one / 3, xx[0] + 0.01, yy[9])
    assert st == oracle.SOURCE_ON_BOUNDARY


def test_weno3_homogeneous(oracle):
    """WENO3 multiplicative: homogeneous Cartesian medium converges to T0."""
    nx, ny = 40, 36
    xx, yy = np.arange(nx) * 0.1, np.arange(ny) * 0.1
    a = np.ones((nx, ny))
    T, st, it = oracle.fsm_weno3_ps_multi_2d(xx, yy, a, a, 0 * a, a / 2.0, 1.73, 1.41)
    assert st == 0
    X, Y = np.meshgrid(xx, yy, indexing="ij")
    ref = np.hypot(X - 1.73, Y - 1.41) / 2.0
    assert rel_pointwise(T, ref) <= 1e-6


# ---------------------------------------------------------------------------
# gaussian_smooth_geo_2 (src/shared/utils.f90:1194-1225)
# ---------------------------------------------------------------------------
_PI_S = float(np.float32(3.14159265359))  # shared_par.f90 pi: a REAL(4) literal


def _smooth_numpy(data, lons, lats, sigma):
    """Second restatement of gaussian_smooth_geo_2, written as the reference's
    array expression: per cell, meshgrid of the clamped window, gps2dist_2
    (utils.f90:1280-1294), w = exp(-delta^2/(2 sigma^2)), sum(w*data)/sum(w)."""
    nx, ny = data.shape
    deg2rad = _PI_S / 180.0
    km2deg = 1.0 / (6371.0 * _PI_S / 180.0)
    sigma3, sigma_sq = sigma * 3, sigma ** 2
    dx, dy = lons[1] - lons[0], lats[1] - lats[0]
    nxw = int(sigma3 / dx)
    out = np.zeros_like(data)
    for j in range(ny):
        nyw = int(sigma3 / math.cos(lats[j] * (math.pi / 180.0)) / dy)
        for i in range(nx):
            m1, m2 = max(0, i - nxw), min(nx - 1, i + nxw)
            n1, n2 = max(0, j - nyw), min(ny - 1, j + nyw)
            lolo, lala = np.meshgrid(lons[m1:m2 + 1], lats[n1:n2 + 1], indexing="ij")
            dlat = (lats[j] - lala) * deg2rad
            dlon = (lolo - lons[i]) * deg2rad
            a = np.sin(dlat * 0.5) ** 2 + np.sin(dlon * 0.5) ** 2 * np.cos(lats[j] * deg2rad) * \
                np.cos(lala * deg2rad)
            delta = 6371.0 * (2.0 * np.arctan2(np.sqrt(a), np.sqrt(1.0 - a))) * km2deg
            w = np.exp(-delta ** 2 / (2.0 * sigma_sq))
            out[i, j] = np.sum(w * data[m1:m2 + 1, n1:n2 + 1]) / np.sum(w)
    return out


def _smooth_grid(nx, ny, x0=100.0, y0=30.0, d=0.05):
    return x0 + d * np.arange(nx), y0 + d * np.arange(ny)


def test_smooth_matches_array_restatement(oracle):
    lons, lats = _smooth_grid(23, 19)
    rng = np.random.default_rng(5)
    data = rng.standard_normal((23, 19))
    got = oracle.gaussian_smooth_geo_2(data, lons, lats, 0.12)
    ref = _smooth_numpy(data, lons, lats, 0.12)
    assert rel_max(got, ref) <= 1e-13


def test_smooth_constant_field(oracle):
    lons, lats = _smooth_grid(31, 27, y0=-10.0, d=0.02)
    got = oracle.gaussian_smooth_geo_2(np.full((31, 27), 2.5), lons, lats, 0.07)
    assert np.max(np.abs(got - 2.5)) <= 1e-13


def test_smooth_window_truncation(oracle):
    """The x half-width is the integer truncation of 3 sigma / dx: a spike at
    column c reaches exactly the columns |i - c| <= int(3 sigma / dx)."""
    lons, lats = _smooth_grid(41, 9, d=0.05)
    sigma = 0.1
    nxw = int(sigma * 3 / (lons[1] - lons[0]))
    spike = np.zeros((41, 9))
    spike[20, 4] = 1.0
    got = oracle.gaussian_smooth_geo_2(spike, lons, lats, sigma)
    cols = np.nonzero(got[:, 4])[0]
    assert cols.min() == 20 - nxw and cols.max() == 20 + nxw
