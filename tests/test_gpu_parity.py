"""CUDA path vs the oracle on the same seeded inputs (GPU only).

Tolerances (plain FP64 path, from the parity contract): travel times and
misfit relative error <= 1e-6, adjoint fields and kernels norm-wise relative
error <= 1e-5.  The FP32-factored path: travel times <= 1e-5, kernels <= 1e-3.
"""
import numpy as np
import pytest

from conftest import rel_max, rel_pointwise
from surfatt_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TT_TOL = 1e-6
KER_TOL = 1e-5
TT_TOL_F32 = 1e-5
KER_TOL_F32 = 1e-3


def _flat(nx, ny, vel=3.0, pert=0.06, x0=100.0, y0=22.0, d=0.05):
    xx, yy = W.arange_grid(x0, nx, d), W.arange_grid(y0, ny, d)
    one = np.ones((nx, ny))
    sv = vel * W.checkerboard_2d(nx, ny, 2, 3, pert)
    return xx, yy, one, one.copy(), np.zeros((nx, ny)), 1.0 / sv


@pytest.mark.parametrize("nx,ny,src", [(41, 41, (101.03, 23.01)), (33, 17, (100.61, 22.37)),
                                       (8, 8, (100.17, 22.18)), (64, 48, (101.5, 23.2))])
def test_forward_lonlat_dropin(sg, oracle, nx, ny, src):
    xx, yy, a, b, c, fun = _flat(nx, ny)
    T, st, it = sg.fsm_uw_ps_lonlat_2d(xx, yy, a, b, c, fun, *src)
    Tr, sr, ir = oracle.fsm_uw_ps_lonlat_2d(xx, yy, a, b, c, fun, *src)
    assert st == sr == 0
    assert it == ir
    assert rel_pointwise(T, Tr) <= TT_TOL


@pytest.mark.parametrize("nx,ny,src", [(200, 150, (103.1, 24.3)), (270, 40, (105.2, 22.9))])
def test_forward_lonlat_dropin_large_grids(sg, oracle, nx, ny, src):
    """A grid whose tau does not fit one block's shared memory (200 x 150)
    runs on the one-block kernel, a long thin one (270 x 40) on the cluster
    forward; both within the tolerance and with the oracle's iteration
    count."""
    xx, yy, a, b, c, fun = _flat(nx, ny, d=0.04)
    T, st, it = sg.fsm_uw_ps_lonlat_2d(xx, yy, a, b, c, fun, *src)
    Tr, sr, ir = oracle.fsm_uw_ps_lonlat_2d(xx, yy, a, b, c, fun, *src)
    assert st == sr == 0
    assert it == ir
    assert rel_pointwise(T, Tr) <= TT_TOL


def test_forward_lonlat_topography_metric(sg, oracle):
    xx, yy, topo, m11, m12, m22 = W.config5_model(n_lon=60, n_lat=50, d=0.02)
    sv = 3.2 * W.checkerboard_2d(60, 50, 2, 2, 0.05)
    src = (xx[25] + 0.007, yy[20] + 0.004)
    T, st, it = sg.fsm_uw_ps_lonlat_2d(xx, yy, m11, m22, -m12, 1.0 / sv, *src)
    Tr, sr, ir = oracle.fsm_uw_ps_lonlat_2d(xx, yy, m11, m22, -m12, 1.0 / sv, *src)
    assert st == sr == 0 and it == ir
    assert rel_pointwise(T, Tr) <= TT_TOL


def test_forward_source_on_boundary(sg, oracle):
    xx, yy, a, b, c, fun = _flat(20, 20)
    sg.set_exit_on_boundary(False)
    T, st, _ = sg.fsm_uw_ps_lonlat_2d(xx, yy, a, b, c, fun, xx[0] + 0.01, yy[10])
    _, sr, _ = oracle.fsm_uw_ps_lonlat_2d(xx, yy, a, b, c, fun, xx[0] + 0.01, yy[10])
    assert st == sr == sg.SOURCE_ON_BOUNDARY


def test_adjoint_lonlat_dropin(sg, oracle):
    xx, yy, a, b, c, fun = _flat(45, 39)
    src = (101.07, 22.93)
    Tr, _, _ = oracle.fsm_uw_ps_lonlat_2d(xx, yy, a, b, c, fun, *src)
    rng = np.random.default_rng(5)
    xr = rng.uniform(xx[2], xx[-3], 12)
    yr = rng.uniform(yy[2], yy[-3], 12)
    sadj = rng.normal(0, 1.0, 12)
    Ta, st, it = sg.fsm_o1_jse_lonlat_2d(xx, yy, a, b, c, Tr, xr, yr, sadj)
    Tar, sr, ir = oracle.fsm_o1_jse_lonlat_2d(xx, yy, a, b, c, Tr, xr, yr, sadj)
    assert st == sr == 0 and it == ir
    assert rel_max(Ta, Tar) <= KER_TOL


def test_adjoint_no_receivers(sg, oracle):
    xx, yy, a, b, c, fun = _flat(20, 18)
    Tr, _, _ = oracle.fsm_uw_ps_lonlat_2d(xx, yy, a, b, c, fun, 100.47, 22.41)
    e = np.zeros(0)
    Ta, st, it = sg.fsm_o1_jse_lonlat_2d(xx, yy, a, b, c, Tr, e, e, e)
    Tar, sr, ir = oracle.fsm_o1_jse_lonlat_2d(xx, yy, a, b, c, Tr, e, e, e)
    assert st == sr and it == ir
    assert np.array_equal(Ta, Tar)


def test_dropins_from_concurrent_threads(sg):
    """Callers on several host threads (the reference's MPI ranks sharing a
    GPU): each thread's forward, adjoint and mask on its own grid give the
    bits the same calls give alone, and each thread reads its own status."""
    from concurrent.futures import ThreadPoolExecutor

    def job(k):
        nx, ny = 24 + 5 * k, 20 + 3 * k
        xx, yy, a, b, c, fun = _flat(nx, ny)
        src = (xx[nx // 3] + 0.013, yy[ny // 2] + 0.021)
        T, st, it = sg.fsm_uw_ps_lonlat_2d(xx, yy, a, b, c, fun, *src)
        xr, yr = xx[[2, nx - 3, nx // 2]], yy[[ny - 3, 2, ny // 2 + 1]]
        Ta, sta, ita = sg.fsm_o1_jse_lonlat_2d(xx, yy, a, b, c, T, xr, yr,
                                               np.array([0.5, -1.0, 0.25]))
        Ta = sg.mask(xx, yy, Ta, *src)
        return T, Ta, (st, it, sta, ita)

    alone = [job(k) for k in range(8)]
    with ThreadPoolExecutor(max_workers=8) as ex:
        for _ in range(2):
            mixed = list(ex.map(job, range(8)))
            for (T, Ta, s), (T0, Ta0, s0) in zip(mixed, alone):
                assert s == s0 and s[0] == sg.OK and s[2] == sg.OK
                assert np.array_equal(T, T0) and np.array_equal(Ta, Ta0)


def test_mask_dropin(sg, oracle):
    xx, yy = W.arange_grid(100, 30, 0.05), W.arange_grid(22, 25, 0.05)
    t = np.random.default_rng(1).normal(size=(30, 25))
    assert np.array_equal(sg.mask(xx, yy, t, 100.52, 22.61), oracle.mask(xx, yy, t, 100.52, 22.61))


@pytest.mark.parametrize("nx,ny,src", [(40, 36, (1.03, 1.21)), (25, 31, (0.55, 0.91))])
def test_forward_cart_dropin(sg, oracle, nx, ny, src):
    xx, yy = np.arange(nx) * 0.05, np.arange(ny) * 0.05
    a = np.ones((nx, ny)) * 1.1
    b = np.ones((nx, ny)) * 0.9
    c = np.full((nx, ny), 0.1)
    fun = 1.0 / (3.0 * W.checkerboard_2d(nx, ny, 2, 2, 0.05))
    T, st, it = sg.fsm_uw_ps_cart_2d(xx, yy, a, b, c, fun, *src)
    Tr, sr, ir = oracle.fsm_uw_ps_cart_2d(xx, yy, a, b, c, fun, *src)
    assert st == sr == 0 and it == ir
    assert rel_pointwise(T, Tr) <= TT_TOL


@pytest.mark.parametrize("name", ["fsm_weno3_ps_multi_2d", "fsm_weno3_ps_2d"])
def test_weno3_dropin(sg, oracle, name):
    nx, ny = 36, 30
    xx, yy = np.arange(nx) * 0.1, np.arange(ny) * 0.1
    a = np.ones((nx, ny))
    b = np.ones((nx, ny))
    c = np.zeros((nx, ny))
    fun = 1.0 / (2.0 * W.checkerboard_2d(nx, ny, 1, 1, 0.05))
    src = (1.73, 1.41)
    T, st, it = getattr(sg, name)(xx, yy, a, b, c, fun, *src)
    Tr, sr, ir = getattr(oracle, name)(xx, yy, a, b, c, fun, *src)
    assert st == sr
    assert abs(it - ir) <= 1
    assert rel_pointwise(T, Tr) <= TT_TOL


def test_cart_adjoint_dropin(sg, oracle):
    nx, ny = 30, 28
    xx, yy = np.arange(nx) * 0.05, np.arange(ny) * 0.05
    a = np.ones((nx, ny))
    b = np.ones((nx, ny))
    c = np.zeros((nx, ny))
    fun = 1.0 / (3.0 * W.checkerboard_2d(nx, ny, 2, 2, 0.05))
    Tr, _, _ = oracle.fsm_uw_ps_cart_2d(xx, yy, a, b, c, fun, 0.71, 0.66)
    xr, yr = np.array([0.2, 1.2, 0.33]), np.array([0.3, 1.1, 1.2])
    s = np.array([0.5, -1.0, 2.0])
    Ta, st, it = sg.fsm_o1_jse_2d(xx, yy, a, b, c, Tr, xr, yr, s)
    Tar, sr, ir = oracle.fsm_o1_jse_2d(xx, yy, a, b, c, Tr, xr, yr, s)
    assert st == sr == 0 and it == ir
    assert rel_max(Ta, Tar) <= KER_TOL


def test_measadj_layer(sg, oracle):
    pb = W.flat_case(nx=40, ny=34, nsta=6, nperiod=1)
    xx, yy = pb.grid(0)
    v, m11, m12, m22 = (pb.field(n, 0) for n in ("svel", "m11", "m12", "m22"))
    s, r0, nr = 2, int(pb.rec_off[2]), int(pb.nrec[2])
    sl = slice(r0, r0 + nr)
    ma = sg.MeasAdj(xx, yy, pb.srcx[s], pb.srcy[s], pb.recx[sl], pb.recy[sl], pb.tt[sl],
                    pb.weight[sl])
    ma.run_forward(v, m11, m22, m12)
    T = np.zeros((40, 34), order="F")
    tek = np.zeros(nr)
    chi = np.zeros(1)
    import ctypes
    lib = oracle.lib()
    it = ctypes.c_int(0)
    D = lambda a: np.asfortranarray(a, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    args = [np.asfortranarray(x, dtype=np.float64) for x in (v, m11, m22, m12)]
    rx, ry, tt, w = (np.ascontiguousarray(x) for x in (pb.recx[sl], pb.recy[sl], pb.tt[sl], pb.weight[sl]))
    lib.orc_run_forward(D(xx), D(yy), 40, 34, D(args[0]), D(args[1]), D(args[2]), D(args[3]),
                        ctypes.c_double(pb.srcx[s]), ctypes.c_double(pb.srcy[s]), nr, D(rx), D(ry),
                        D(tt), D(w), D(T), D(tek), D(chi), ctypes.byref(it))
    assert rel_pointwise(ma.timetable, T) <= TT_TOL
    assert rel_pointwise(ma.tekio, tek) <= TT_TOL
    assert abs(ma.chi - chi[0]) <= TT_TOL * abs(chi[0])
    adj = ma.run_adjoint(m11, m22, m12)
    den = ma.run_adjoint_density(m11, m22, m12)
    wr = w.copy()
    adjr = np.zeros((40, 34), order="F")
    denr = np.zeros((40, 34), order="F")
    lib.orc_run_adjoint(D(xx), D(yy), 40, 34, D(args[1]), D(args[2]), D(args[3]),
                        ctypes.c_double(pb.srcx[s]), ctypes.c_double(pb.srcy[s]), nr, D(rx), D(ry),
                        D(tt), D(tek), wr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), D(T),
                        D(adjr), ctypes.byref(it))
    lib.orc_run_adjoint_density(D(xx), D(yy), 40, 34, D(args[1]), D(args[2]), D(args[3]),
                                ctypes.c_double(pb.srcx[s]), ctypes.c_double(pb.srcy[s]), nr,
                                D(rx), D(ry), wr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                D(T), D(denr), ctypes.byref(it))
    assert np.array_equal(ma.weight, wr)
    assert rel_max(adj, adjr) <= KER_TOL
    assert rel_max(den, denr) <= KER_TOL


def _engine_vs_oracle(sg, oracle, pb, mode, prec, tt_tol, ker_tol):
    eng = sg.Engine(0)
    got = eng.evaluate(pb, mode=mode, precision=prec)
    ref = oracle.gradient_eval(pb, mode=mode, nthreads=4)
    assert np.all(got["status"] == ref["status"])
    assert rel_pointwise(got["tt_fwd"], ref["tt_fwd"]) <= tt_tol
    assert abs(got["chi"] - ref["chi"]) <= tt_tol * 10 * abs(ref["chi"])
    if mode >= 2:
        for p in range(pb.nperiod):
            g0, n = int(pb.goff[p]), int(pb.nx[p] * pb.ny[p])
            assert rel_max(got["adj_s"][g0:g0 + n], ref["adj_s"][g0:g0 + n]) <= ker_tol, p
            if mode == 3:
                assert rel_max(got["adj_density"][g0:g0 + n],
                               ref["adj_density"][g0:g0 + n]) <= ker_tol, p
    if prec == sg.PREC_FP64:
        assert np.all(np.abs(got["fwd_iters"] - ref["fwd_iters"]) <= 0)
    eng.close()
    return got, ref


@pytest.mark.parametrize("mode", [0, 2, 3])
def test_engine_fp64_flat(sg, oracle, mode):
    pb = W.flat_case(nx=50, ny=44, nsta=6, nperiod=2, mode=mode)
    _engine_vs_oracle(sg, oracle, pb, mode, sg.PREC_FP64, TT_TOL, KER_TOL)


def test_engine_fp64_config1(sg, oracle):
    import os
    from conftest import GOLDEN
    obs = W.read_src_rec_tt(os.path.join(GOLDEN, "config1_src_rec.csv"))
    pb = W.config1(observed_tt=obs)
    _engine_vs_oracle(sg, oracle, pb, 2, sg.PREC_FP64, TT_TOL, KER_TOL)


def test_engine_fp32_flat(sg, oracle):
    pb = W.flat_case(nx=60, ny=52, nsta=7, nperiod=2, mode=3)
    _engine_vs_oracle(sg, oracle, pb, 3, sg.PREC_FP32, TT_TOL_F32, KER_TOL_F32)


def test_engine_fp32_four_bands(sg, oracle):
    """FP32 warp-per-solve kernel with four 32-row bands per lane (ny = 120)."""
    pb = W.flat_case(nx=130, ny=120, nsta=5, nperiod=2, mode=3)
    _engine_vs_oracle(sg, oracle, pb, 3, sg.PREC_FP32, TT_TOL_F32, KER_TOL_F32)


def test_engine_fp32_mode2_odd_grid(sg, oracle):
    pb = W.flat_case(nx=71, ny=45, nsta=6, nperiod=1, mode=2)
    _engine_vs_oracle(sg, oracle, pb, 2, sg.PREC_FP32, TT_TOL_F32, KER_TOL_F32)


def test_engine_fp32_tall_grids(sg, oracle):
    """Grids taller than 128 rows: warp teams (automatic) and the
    one-block-per-solve kernel (forced) both match the oracle."""
    pb = W.config4(nsrc=4, nperiod=3, nmax=168, nmin=48, span_deg=2.0)
    _engine_vs_oracle(sg, oracle, pb, 3, sg.PREC_FP32, TT_TOL_F32, KER_TOL_F32)
    ref = oracle.gradient_eval(pb, mode=3, nthreads=8)
    st, kv, out = _run_kernel(sg, pb, 3, 1, -1)
    assert st == sg.OK and kv["kind"] == 1
    assert rel_pointwise(out["tt_fwd"], ref["tt_fwd"]) <= TT_TOL_F32
    assert rel_max(out["adj_s"], ref["adj_s"]) <= KER_TOL_F32


@pytest.mark.parametrize("nx,ny", [(60, 200), (150, 257), (96, 384), (40, 512)])
@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5])
def test_fp32_warp_teams(sg, oracle, nx, ny, variant):
    """Warp teams (2 to 4 warps of 128 rows) and one warp sweeping the same
    row blocks as strips (variants 4, 5): every variant gives the same bits
    and matches the oracle within the FP32 tolerances."""
    pb = W.flat_case(nx=nx, ny=ny, d=0.02, nsta=4, nperiod=1, mode=3, seed=40 + ny)
    st0, kv0, base = _run_kernel(sg, pb, 3, 2, 0)
    st, kv, o = _run_kernel(sg, pb, 3, 2, variant)
    assert st0 == st == sg.OK and kv == dict(kind=2, variant=variant)
    assert np.array_equal(o["tt_fwd"], base["tt_fwd"])
    assert np.array_equal(o["adj_s"], base["adj_s"])
    assert np.array_equal(o["adj_density"], base["adj_density"])
    if variant == 0:
        ref = oracle.gradient_eval(pb, mode=3, nthreads=8)
        assert np.all(o["status"] == ref["status"])
        assert rel_pointwise(o["tt_fwd"], ref["tt_fwd"]) <= TT_TOL_F32
        assert rel_max(o["adj_s"], ref["adj_s"]) <= KER_TOL_F32
        assert rel_max(o["adj_density"], ref["adj_density"]) <= KER_TOL_F32


def test_fp32_team_batch_small_grids_unchanged(sg):
    """In a batch that needs warp teams (one tall grid), the solves on small
    grids give the bits they give alone (single warps)."""
    pb = W.config4(nsrc=5, nperiod=3, nmax=200, nmin=48, span_deg=2.0, seed=41)
    assert int(np.max(pb.ny)) > 128 and int(np.min(pb.ny)) <= 128
    eng = sg.Engine(0)
    full = eng.evaluate(pb, mode=3, precision=sg.PREC_FP32)
    small = [s for s in range(pb.nsolve) if pb.ny[pb.pidx[s]] <= 128][:3]
    for s in small:
        one = eng.evaluate(pb.subset([s]), mode=3, precision=sg.PREC_FP32)
        r0, nr = int(pb.rec_off[s]), int(pb.nrec[s])
        assert np.array_equal(one["tt_fwd"], full["tt_fwd"][pb.path[r0:r0 + nr]])
    eng.close()


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5])
def test_fp32_team_classes(sg, oracle, variant):
    """A batch of three team classes (grids of 48 to 304 rows) runs as one
    concurrent launch per class; every solve gives the bits it gives as
    the only solve of its evaluation, in every variant, and the batch meets
    the FP32 tolerances against the oracle."""
    pb = W.config4(nsrc=4, nperiod=5, nmax=300, nmin=48, span_deg=2.0, seed=42)
    teams = {1 if n <= 128 else (int(n) + 127) // 128 for n in pb.ny}
    assert teams == {1, 2, 3}
    eng = sg.Engine(0)
    eng.load(pb)
    eng.set_kernel(sg.PREC_FP32, kind=2, variant=variant)
    eng.run(3, sg.PREC_FP32)
    assert eng.sync() == sg.OK
    assert eng.timing()[2] == 3 + 2   # three class launches, the kernel sums (both fields), misfit
    full = eng.results()
    eng.close()
    assert np.all(full["status"] == sg.OK)
    for p in range(pb.nperiod):
        s = int(np.flatnonzero(pb.pidx == p)[0])
        st, _, one = _run_kernel(sg, pb.subset([s]), 3, 2, variant)
        r0, nr = int(pb.rec_off[s]), int(pb.nrec[s])
        assert st == sg.OK
        assert np.array_equal(one["tt_fwd"], full["tt_fwd"][pb.path[r0:r0 + nr]])
        assert one["fwd_iters"][0] == full["fwd_iters"][s]
        assert one["adj_iters"][0] == full["adj_iters"][s]
    if variant == 0:
        ref = oracle.gradient_eval(pb, mode=3, nthreads=8)
        assert rel_pointwise(full["tt_fwd"], ref["tt_fwd"]) <= TT_TOL_F32
        assert rel_max(full["adj_s"], ref["adj_s"]) <= KER_TOL_F32
        assert rel_max(full["adj_density"], ref["adj_density"]) <= KER_TOL_F32


def test_engine_fp64_large_grid(sg, oracle):
    """The plain FP64 path on a 220 x 300 grid: anti-diagonals longer than its
    128-thread block, within the plain tolerances."""
    pb = W.flat_case(nx=220, ny=300, d=0.01, nsta=3, nperiod=1, mode=3, seed=18)
    _engine_vs_oracle(sg, oracle, pb, 3, sg.PREC_FP64, TT_TOL, KER_TOL)


def test_engine_fp32_wide_grid_block_kernel(sg, oracle):
    """A grid wider than the row kernel's column limit (4096) runs on the
    block-per-solve kernel, automatically, within the FP32 tolerances."""
    pb = W.flat_case(nx=4104, ny=10, d=0.001, nsta=3, nperiod=1, mode=2, seed=17)
    eng = sg.Engine(0)
    got = eng.evaluate(pb, mode=2, precision=sg.PREC_FP32)
    assert eng.kernel_variant()["kind"] == 1
    eng.close()
    ref = oracle.gradient_eval(pb, mode=2, nthreads=4)
    assert np.all(got["status"] == ref["status"])
    assert rel_pointwise(got["tt_fwd"], ref["tt_fwd"]) <= TT_TOL_F32
    assert rel_max(got["adj_s"], ref["adj_s"]) <= KER_TOL_F32


def test_fp32_single_class_ignores_periods_without_solves(sg):
    """Solves of one team class in a problem that also holds taller grids
    without solves run on their own class's team (two warps for 192 rows,
    not the three a 304-row grid would need) and give the bits they give in
    the full multi-class batch."""
    pb = W.config4(nsrc=4, nperiod=5, nmax=300, nmin=48, span_deg=2.0, seed=42)
    sel = [s for s in range(pb.nsolve) if 128 < pb.ny[pb.pidx[s]] <= 256]
    assert sel and int(np.max(pb.ny)) > 256
    eng = sg.Engine(0)
    full = eng.evaluate(pb, mode=3, precision=sg.PREC_FP32)
    sub = pb.subset(sel)
    eng.load(sub)
    eng.set_kernel(sg.PREC_FP32, kind=2, variant=0)  # teams (automatic: strips)
    eng.run(3, sg.PREC_FP32)
    assert eng.sync() == sg.OK
    assert eng.launch_config()["block"] == 64
    one = eng.results()
    eng.close()
    for q, s in enumerate(sel):
        r0, nr = int(pb.rec_off[s]), int(pb.nrec[s])
        q0 = int(sub.rec_off[q])
        assert np.array_equal(one["tt_fwd"][q0:q0 + nr], full["tt_fwd"][pb.path[r0:r0 + nr]])


def _drop_receivers(pb, solves):
    """The problem with the receiver lists of `solves` emptied (the other
    solves keep theirs and their path indices)."""
    import dataclasses
    offs, nrec, keep = [], [], []
    for s in range(pb.nsolve):
        r0, n = int(pb.rec_off[s]), 0 if s in solves else int(pb.nrec[s])
        offs.append(len(keep))
        nrec.append(n)
        keep.extend(range(r0, r0 + n))
    ridx = np.asarray(keep, np.int64)
    return dataclasses.replace(
        pb, rec_off=np.asarray(offs, np.int32), nrec=np.asarray(nrec, np.int32),
        recx=pb.recx[ridx].copy(), recy=pb.recy[ridx].copy(), tt=pb.tt[ridx].copy(),
        weight=pb.weight[ridx].copy(), path=pb.path[ridx].copy(), n_paths=pb.npath)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_engine_solves_without_receivers(sg, oracle, prec):
    """Solves with empty receiver lists (zero misfit, zero adjoint sources),
    among solves with receivers, on a one-warp grid and on a team grid."""
    P = sg.PREC_FP64 if prec == "fp64" else sg.PREC_FP32
    tols = (TT_TOL, KER_TOL) if prec == "fp64" else (TT_TOL_F32, KER_TOL_F32)
    pb = _drop_receivers(W.flat_case(nx=40, ny=36, nsta=5, nperiod=2, mode=3, seed=13), {0, 3})
    assert pb.nrec[0] == 0 and pb.nrec[3] == 0 and pb.nrec[1] > 0
    _engine_vs_oracle(sg, oracle, pb, 3, P, *tols)
    pb = _drop_receivers(W.flat_case(nx=30, ny=150, d=0.02, nsta=4, nperiod=1, mode=3,
                                     seed=14), {1})
    _engine_vs_oracle(sg, oracle, pb, 3, P, *tols)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_engine_empty_work_list(sg, prec):
    """No solves: zero kernels and misfit, every launch still well formed."""
    P = sg.PREC_FP64 if prec == "fp64" else sg.PREC_FP32
    pb = W.flat_case(nx=30, ny=28, nsta=4, nperiod=2, mode=3, seed=15).subset([])
    assert pb.nsolve == 0
    eng = sg.Engine(0)
    got = eng.evaluate(pb, mode=3, precision=P)
    eng.close()
    assert got["chi"] == 0.0
    assert not np.any(got["adj_s"]) and not np.any(got["adj_density"])


def test_engine_fp32_team_source_on_boundary(sg, oracle):
    """A source on the grid boundary of a team grid (200 rows): that solve
    reports it and contributes nothing; the others match the oracle."""
    pb = W.flat_case(nx=40, ny=200, d=0.02, nsta=4, nperiod=1, mode=2, seed=16)
    xx, _ = pb.grid(0)
    pb.srcx[2] = xx[-1] - 0.001
    eng = sg.Engine(0)
    got = eng.evaluate(pb, mode=2, precision=sg.PREC_FP32)
    eng.close()
    ref = oracle.gradient_eval(pb, mode=2, nthreads=4)
    assert got["status"][2] == sg.SOURCE_ON_BOUNDARY == ref["status"][2]
    assert np.all(got["status"] == ref["status"])
    assert rel_max(got["adj_s"], ref["adj_s"]) <= KER_TOL_F32


def test_engine_uneven_grids(sg, oracle):
    pb = W.config4(nsrc=5, nperiod=3, nmax=72, nmin=40, span_deg=2.0)
    _engine_vs_oracle(sg, oracle, pb, 3, sg.PREC_FP64, TT_TOL, KER_TOL)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_engine_many_periods(sg, oracle, prec):
    """40 periods: the per-period precompute runs in two launches (32 + 8)."""
    pb = W.config4(nsrc=3, nperiod=40, nmax=40, nmin=24, span_deg=2.0)
    assert pb.nperiod == 40
    if prec == "fp64":
        _engine_vs_oracle(sg, oracle, pb, 3, sg.PREC_FP64, TT_TOL, KER_TOL)
    else:
        _engine_vs_oracle(sg, oracle, pb, 3, sg.PREC_FP32, TT_TOL_F32, KER_TOL_F32)


def test_batched_equals_single_solves(sg):
    """Every solve's result is independent of the batch it runs in."""
    pb = W.flat_case(nx=40, ny=36, nsta=6, nperiod=2, mode=3)
    eng = sg.Engine(0)
    full = eng.evaluate(pb, mode=3)
    for s in (0, 7, pb.nsolve - 1):
        sub = pb.subset([s])
        one = eng.evaluate(sub, mode=3)
        r0, nr = int(pb.rec_off[s]), int(pb.nrec[s])
        assert np.array_equal(one["tt_fwd"], full["tt_fwd"][pb.path[r0:r0 + nr]])
    eng.close()


def test_engine_source_on_boundary_status(sg, oracle):
    pb = W.flat_case(nx=30, ny=30, nsta=4, nperiod=1, mode=2)
    xx, _ = pb.grid(0)
    pb.srcx[1] = xx[0] + 0.001
    eng = sg.Engine(0)
    got = eng.evaluate(pb, mode=2)
    ref = oracle.gradient_eval(pb, mode=2)
    assert got["status"][1] == sg.SOURCE_ON_BOUNDARY == ref["status"][1]
    assert rel_max(got["adj_s"], ref["adj_s"]) <= KER_TOL
    eng.close()


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5])
def test_fp32_warp_variants(sg, oracle, variant):
    """Every warp-kernel variant agrees with the oracle within the FP32
    tolerances, and all variants give the same bits (they differ only in when
    operands are loaded and in register allocation)."""
    pb = W.flat_case(nx=100, ny=90, nsta=6, nperiod=2, mode=3, seed=31)
    ref = oracle.gradient_eval(pb, mode=3, nthreads=4)
    eng = sg.Engine(0)
    eng.load(pb)
    eng.set_kernel(sg.PREC_FP32, kind=2, variant=0)
    eng.run(3, sg.PREC_FP32)
    assert eng.sync() == sg.OK
    base = eng.results()
    eng.set_kernel(sg.PREC_FP32, kind=2, variant=variant)
    eng.run(3, sg.PREC_FP32)
    assert eng.sync() == sg.OK
    assert eng.kernel_variant() == dict(kind=2, variant=variant)
    o = eng.results()
    assert np.array_equal(o["tt_fwd"], base["tt_fwd"])
    assert np.array_equal(o["adj_s"], base["adj_s"])
    assert np.array_equal(o["adj_density"], base["adj_density"])
    assert np.all(o["status"] == ref["status"])
    assert rel_pointwise(o["tt_fwd"], ref["tt_fwd"]) <= TT_TOL_F32
    for p in range(pb.nperiod):
        sl = slice(int(pb.goff[p]), int(pb.goff[p] + pb.nx[p] * pb.ny[p]))
        assert rel_max(o["adj_s"][sl], ref["adj_s"][sl]) <= KER_TOL_F32
        assert rel_max(o["adj_density"][sl], ref["adj_density"][sl]) <= KER_TOL_F32
    eng.close()


def test_forced_kernels_reject_too_tall_grids(sg):
    """The row kernel takes 512 rows (teams); forcing it on a taller grid
    fails the run, the automatic choice (block kernel) runs; an unknown
    kernel kind is rejected."""
    pb = W.flat_case(nx=20, ny=520, d=0.01, nsta=3, nperiod=1, mode=2, seed=32)
    eng = sg.Engine(0)
    eng.load(pb)
    eng.set_kernel(sg.PREC_FP32, kind=2)
    with pytest.raises(sg.SurfattError):
        eng.run(2, sg.PREC_FP32)
    eng.set_kernel(sg.PREC_FP32)
    eng.run(2, sg.PREC_FP32)
    assert eng.sync() == sg.OK
    with pytest.raises(sg.SurfattError):
        eng.set_kernel(sg.PREC_FP32, kind=3)
    eng.close()


def _run_kernel(sg, pb, mode, kind, variant):
    eng = sg.Engine(0)
    eng.load(pb)
    eng.set_kernel(sg.PREC_FP32, kind=kind, variant=variant)
    eng.run(mode, sg.PREC_FP32)
    st = eng.sync()
    kv = eng.kernel_variant()
    out = eng.results()
    eng.close()
    return st, kv, out


@pytest.mark.parametrize("case", ["square", "mixed", "mode2", "mode0"])
def test_fp32_row_kernel_items_and_whole_solves(sg, oracle, case):
    """The row kernel with solves cut into work items and with whole solves
    gives the same bits (same visits in the same order) in every mode, on
    one grid and on uneven grids of one evaluation, and meets the FP32
    tolerances against the oracle."""
    if case == "mixed":
        pb = W.config4(nsrc=3, nperiod=4, nmax=120, nmin=36, span_deg=2.0)
        mode = 3
    else:
        mode = {"square": 3, "mode2": 2, "mode0": 0}[case]
        pb = W.flat_case(nx=97, ny=75, nsta=5, nperiod=2, mode=mode, seed=41)
    st_i, kv_i, d = _run_kernel(sg, pb, mode, 2, 0)
    st_w, kv_w, w = _run_kernel(sg, pb, mode, 2, 1)
    assert kv_i == dict(kind=2, variant=0) and kv_w == dict(kind=2, variant=1)
    assert st_i == st_w
    assert np.array_equal(d["status"], w["status"])
    assert np.array_equal(d["fwd_iters"], w["fwd_iters"])
    assert np.array_equal(d["tt_fwd"], w["tt_fwd"])
    if mode >= 2:
        assert np.array_equal(d["adj_iters"], w["adj_iters"])
        for key in ("adj_s", "adj_density") if mode == 3 else ("adj_s",):
            assert np.array_equal(d[key], w[key]), (key, rel_max(d[key], w[key]))
    ref = oracle.gradient_eval(pb, mode=mode, nthreads=4)
    assert np.all(d["status"] == ref["status"])
    assert rel_pointwise(d["tt_fwd"], ref["tt_fwd"]) <= TT_TOL_F32
    if mode >= 2:
        for p in range(pb.nperiod):
            sl = slice(int(pb.goff[p]), int(pb.goff[p] + pb.nx[p] * pb.ny[p]))
            assert rel_max(d["adj_s"][sl], ref["adj_s"][sl]) <= KER_TOL_F32
            if mode == 3:
                assert rel_max(d["adj_density"][sl], ref["adj_density"][sl]) <= KER_TOL_F32


def test_fp64_work_items_equal_whole_solves(sg, oracle):
    """The plain FP64 kernel cut into work items (the engine's default:
    forward items of two iterations, then the rest of the solve; only tau
    kept per solve between items) gives the bits of the whole-solve kernel,
    on uneven grids with a boundary source and solves that converge inside
    an early item, and matches the oracle."""
    pb = W.config4(nsrc=5, nperiod=4, nmax=96, nmin=24, span_deg=2.0, seed=44)
    eng = sg.Engine(0)
    eng.load(pb)
    eng.set_kernel(sg.PREC_FP64, kind=0, variant=1)
    whole = eng.evaluate(mode=3, precision=sg.PREC_FP64)
    eng.set_kernel(sg.PREC_FP64, kind=0, variant=0)
    cut = eng.evaluate(mode=3, precision=sg.PREC_FP64)
    assert eng.kernel_variant() == dict(kind=0, variant=0)
    for k in ("adj_s", "adj_density", "tt_fwd", "status", "fwd_iters", "adj_iters"):
        assert np.array_equal(cut[k], whole[k]), k
    assert cut["chi"] == whole["chi"]
    ref = oracle.gradient_eval(pb, mode=3, nthreads=8)
    assert np.array_equal(cut["status"], ref["status"])
    assert np.array_equal(cut["fwd_iters"], ref["fwd_iters"])
    assert rel_pointwise(cut["tt_fwd"], ref["tt_fwd"]) <= TT_TOL
    assert rel_max(cut["adj_s"], ref["adj_s"]) <= KER_TOL
    eng.close()
