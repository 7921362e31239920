"""Kernel combination and multigrid projection on the GPU vs the oracle
(GPU only).

The CUDA kernels keep the reference's summation orders, its association of
every product and its walking search's tie resolution, with explicitly
rounded FP64 operations, so the comparisons are bitwise
(np.array_equal); the density preconditioner (kdensity_coe > 0) calls the
device's pow(), so that case is compared to 1e-13 norm-wise.
"""
import numpy as np
import pytest

from conftest import rel_max
from surfatt_gb300 import workloads as W
from test_oracle_project import tie_grids

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("abr,rs", [(False, False), (True, False), (True, True)])
def test_combine_bitwise(sg, oracle, abr, rs):
    k = W.kernel3d_case(nx=23, ny=19, nz=11, nperiod=5, seed=7)
    got = sg.combine_kernels(k.adj_s, k.adj_density, k.sen_vs, k.sen_vp, k.sen_rho, k.vs3d,
                             k.vp3d, abr, rs)
    ref = oracle.combine_kernels(k.adj_s, k.adj_density, k.sen_vs, k.sen_vp, k.sen_rho, k.vs3d,
                                 k.vp3d, abr, rs)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])


def test_projection_dropins_bitwise_with_ties(sg, oracle):
    vx, vy, vz, xinv, yinv, zinv = tie_grids()
    rng = np.random.default_rng(8)
    adj = np.asfortranarray(rng.standard_normal((7, 6, 5)))
    gk = sg.inv_grid_iso(xinv, yinv, zinv, adj, vx, vy, vz)
    assert np.array_equal(gk, oracle.inv_grid_iso(xinv, yinv, zinv, adj, vx, vy, vz))
    g2 = rng.standard_normal(gk.shape)
    up = sg.inv2fwd_iso(xinv, yinv, zinv, g2, vx, vy, vz)
    assert np.array_equal(up, oracle.inv2fwd_iso(xinv, yinv, zinv, g2, vx, vy, vz))


@pytest.mark.parametrize("shape,ninv,nset", [((60, 60, 30), (8, 9, 8), 5),
                                             ((31, 17, 9), (6, 5, 4), 3),
                                             ((12, 40, 25), (5, 10, 9), 1)])
def test_projection_dropins_bitwise(sg, oracle, shape, ninv, nset):
    nx, ny, nz = shape
    k = W.kernel3d_case(nx=nx, ny=ny, nz=nz, nperiod=1, n_inv_grid=ninv, nset=nset)
    rng = np.random.default_rng(9)
    adj = np.asfortranarray(rng.standard_normal(shape))
    gk = sg.inv_grid_iso(k.xinv, k.yinv, k.zinv, adj, k.xgrids, k.ygrids, k.zgrids)
    gr = oracle.inv_grid_iso(k.xinv, k.yinv, k.zinv, adj, k.xgrids, k.ygrids, k.zgrids)
    assert np.array_equal(gk, gr)
    up = sg.inv2fwd_iso(k.xinv, k.yinv, k.zinv, gr, k.xgrids, k.ygrids, k.zgrids)
    assert np.array_equal(up, oracle.inv2fwd_iso(k.xinv, k.yinv, k.zinv, gr, k.xgrids,
                                                 k.ygrids, k.zgrids))


def test_post_process_bitwise(sg, oracle):
    k = W.kernel3d_case(nx=30, ny=28, nz=14, nperiod=4, seed=10)
    ker, kd = oracle.combine_kernels(k.adj_s, k.adj_density, k.sen_vs, k.sen_vp, k.sen_rho,
                                     k.vs3d, k.vp3d, True, False)
    g0 = np.asfortranarray(np.random.default_rng(11).standard_normal(ker.shape))
    got = sg.post_process_kernels(ker, kd, 0.0, k.xinv, k.yinv, k.zinv, k.xgrids, k.ygrids,
                                  k.zgrids, k.chi0, 0.7, g0)
    ref = oracle.post_process_kernels(ker, kd, 0.0, k.xinv, k.yinv, k.zinv, k.xgrids, k.ygrids,
                                      k.zgrids, k.chi0, 0.7, g0)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])


@pytest.mark.parametrize("coe", [0.5, 1.0])
def test_post_process_preconditioned(sg, oracle, coe):
    k = W.kernel3d_case(nx=30, ny=28, nz=14, nperiod=4, seed=12)
    ker, kd = oracle.combine_kernels(k.adj_s, k.adj_density, k.sen_vs, k.sen_vp, k.sen_rho,
                                     k.vs3d, k.vp3d, True, True)
    kd = kd.copy(order="F")
    kd[:, 5, 5, 5] = 0.0     # below the threshold: preconditioner 0
    g0 = np.zeros_like(ker)
    got = sg.post_process_kernels(ker, kd, coe, k.xinv, k.yinv, k.zinv, k.xgrids, k.ygrids,
                                  k.zgrids, k.chi0, 1.0, g0)
    ref = oracle.post_process_kernels(ker, kd, coe, k.xinv, k.yinv, k.zinv, k.xgrids, k.ygrids,
                                      k.zgrids, k.chi0, 1.0, g0)
    assert np.array_equal(got[0] == 0, ref[0] == 0)
    for q in range(3):
        assert rel_max(got[0][q], ref[0][q]) <= 1e-13
        assert rel_max(got[1][q], ref[1][q]) <= 1e-13


@pytest.mark.parametrize("abr", [False, True])
def test_kernel_gradient_config2_model_bitwise(sg, oracle, abr):
    """The fused call on config 2's model (60 x 60 x 30, 16 periods,
    5 sets of 8 x 9 x 8 inversion nodes) equals the oracle's
    combine_kernels + post_processing_for_kernel bit for bit."""
    k = W.kernel3d_case()
    g0 = np.zeros((3 if abr else 1, 60, 60, 30), order="F")
    ker, kd, grad = sg.kernel_gradient(k, use_alpha_beta_rho=abr, gradient_s=g0)
    rk, rkd = oracle.combine_kernels(k.adj_s, k.adj_density, k.sen_vs, k.sen_vp, k.sen_rho,
                                     k.vs3d, k.vp3d, abr, False)
    rk2, rg = oracle.post_process_kernels(rk, rkd, 0.0, k.xinv, k.yinv, k.zinv, k.xgrids,
                                          k.ygrids, k.zgrids, k.chi0, k.weight, g0)
    assert np.array_equal(ker, rk2) and np.array_equal(kd, rkd) and np.array_equal(grad, rg)
    ms, n = sg.kernel_gradient_timing()
    assert ms > 0 and n == 5


def test_projection_not_located_raises(sg):
    vx, vy, vz, xinv, yinv, zinv = tie_grids(nset=1)
    xinv = xinv.copy(order="F")
    xinv[0, 0] = 0.5
    sg.set_exit_on_boundary(False)
    try:
        with pytest.raises(sg.SurfattError):
            sg.inv2fwd_iso(xinv, yinv, zinv, np.zeros(64), vx, vy, vz)
        # a located call on the same thread afterwards works
        gk = sg.inv_grid_iso(xinv, yinv, zinv, np.ones((7, 6, 5)), vx, vy, vz)
        assert np.isfinite(gk).all()
    finally:
        sg.set_exit_on_boundary(True)
