"""Pins of the oracle's kernel combination and multigrid projection (no GPU).

The reference has no tests for these routines and cannot be built here, so
the C restatement in oracle/oracle_project.c is pinned by a second, literal
pure-Python restatement on small grids (including model nodes that lie
exactly on inversion-grid planes, where the walking search's direction
matters), by conservation and linear-reproduction identities, and by the
inversion-grid construction restated in surfatt_gb300.workloads.
"""
import numpy as np
import pytest

from conftest import rel_max
from surfatt_gb300 import workloads as W

F32 = np.float32


# --------------------------------------------------------------------------
# literal restatement (pure Python, 1-based walk state as in the reference)
# --------------------------------------------------------------------------
def _walk(xx, v, i1):
    n = len(v)
    w = None
    while i1 > 0 and i1 < n:
        if xx < v[i1 - 1]:
            i1 -= 1
        elif xx <= v[i1]:
            w = (xx - v[i1 - 1]) / (v[i1] - v[i1 - 1])
            return i1, w
        else:
            i1 += 1
    return i1, w


def _locate(x, y, z, xv, yv, zv, st):
    st[0], wx = _walk(x, xv, st[0])
    st[1], wy = _walk(y, yv, st[1])
    st[2], wz = _walk(z, zv, st[2])
    if wx is None or wy is None or wz is None:
        return None
    o = 1.0
    return [(o - wx) * (o - wy) * (o - wz), (o - wx) * wy * (o - wz), wx * wy * (o - wz),
            wx * (o - wy) * (o - wz), (o - wx) * (o - wy) * wz, (o - wx) * wy * wz,
            wx * wy * wz, wx * (o - wy) * wz]


_DI = [0, 0, 1, 1, 0, 0, 1, 1]
_DJ = [0, 1, 1, 0, 0, 1, 1, 0]
_DK = [0, 0, 0, 0, 1, 1, 1, 1]


def _py_inv_grid(xinv, yinv, zinv, adj, vx, vy, vz):
    nxi, nyi, nzi, nset = xinv.shape[0], yinv.shape[0], zinv.shape[0], xinv.shape[1]
    nx, ny, nz = adj.shape
    dx, dy, dz = vx[1] - vx[0], vy[1] - vy[0], vz[1] - vz[0]
    gk = [0.0] * (nset * nxi * nyi * nzi)
    for s in range(nset):
        st = [1, 1, 1]
        for j in range(1, ny - 1):
            for i in range(1, nx - 1):
                for k in range(1, nz - 1):
                    wt = _locate(vx[i], vy[j], vz[k], xinv[:, s], yinv[:, s], zinv[:, s], st)
                    assert wt is not None
                    for n in range(8):
                        m = s * nxi * nyi * nzi + (st[0] - 1 + _DI[n]) + nxi * (
                            (st[1] - 1 + _DJ[n]) + nyi * (st[2] - 1 + _DK[n]))
                        gk[m] = gk[m] + float(adj[i, j, k]) * dx * dy * dz * wt[n]
    return np.array(gk)


def _py_inv2fwd(xinv, yinv, zinv, gk, vx, vy, vz):
    nxi, nyi, nzi, nset = xinv.shape[0], yinv.shape[0], zinv.shape[0], xinv.shape[1]
    nx, ny, nz = len(vx), len(vy), len(vz)
    upd = np.zeros((nx, ny, nz))
    for s in range(nset):
        st = [1, 1, 1]
        for j in range(ny):
            for i in range(nx):
                for k in range(nz):
                    wt = _locate(vx[i], vy[j], vz[k], xinv[:, s], yinv[:, s], zinv[:, s], st)
                    assert wt is not None
                    val = 0.0
                    for n in range(8):
                        m = s * nxi * nyi * nzi + (st[0] - 1 + _DI[n]) + nxi * (
                            (st[1] - 1 + _DJ[n]) + nyi * (st[2] - 1 + _DK[n]))
                        val = val + wt[n] * float(gk[m])
                    upd[i, j, k] = upd[i, j, k] + val
    return upd


def tie_grids(nset=3):
    """Model axes 0..6, 0..5, 0..4 (unit steps) and inversion grids, shifted
    per set, whose planes pass through model nodes: x = 1, 3 (set 0) and
    2, 4 (set 2); y = 2, 4 (set 0) and 3, 5 (set 2, 5 the last node);
    z = 1, 3 (set 0) and 0, 2, 4 (set 2, the first and last nodes)."""
    vx, vy, vz = np.arange(7.0), np.arange(6.0), np.arange(5.0)
    bx = np.array([-1.5, 1.0, 3.0, 7.5])
    by = np.array([-1.5, 2.0, 4.0, 6.5])
    bz = np.array([-1.0, 1.0, 3.0, 5.0])
    xinv = np.asfortranarray(np.stack([bx + 0.5 * s * (-1) ** s for s in range(nset)], axis=1))
    yinv = np.asfortranarray(np.stack([by + 0.5 * s for s in range(nset)], axis=1))
    zinv = np.asfortranarray(np.stack([bz + 0.5 * s for s in range(nset)], axis=1))
    return vx, vy, vz, xinv, yinv, zinv


def test_projection_matches_literal_walk_with_ties(oracle):
    vx, vy, vz, xinv, yinv, zinv = tie_grids()
    rng = np.random.default_rng(3)
    adj = np.asfortranarray(rng.standard_normal((7, 6, 5)))
    gk = oracle.inv_grid_iso(xinv, yinv, zinv, adj, vx, vy, vz)
    assert np.array_equal(gk, _py_inv_grid(xinv, yinv, zinv, adj, vx, vy, vz))
    g2 = rng.standard_normal(gk.shape)
    up = oracle.inv2fwd_iso(xinv, yinv, zinv, g2, vx, vy, vz)
    assert np.array_equal(up, _py_inv2fwd(xinv, yinv, zinv, g2, vx, vy, vz))


def test_projection_matches_literal_walk_config_like(oracle):
    k = W.kernel3d_case(nx=11, ny=9, nz=7, nperiod=2, d=0.1, zmax=12.0, n_inv_grid=(5, 5, 4),
                        nset=3)
    rng = np.random.default_rng(4)
    adj = np.asfortranarray(rng.standard_normal((11, 9, 7)))
    gk = oracle.inv_grid_iso(k.xinv, k.yinv, k.zinv, adj, k.xgrids, k.ygrids, k.zgrids)
    assert np.array_equal(gk, _py_inv_grid(k.xinv, k.yinv, k.zinv, adj, k.xgrids, k.ygrids,
                                           k.zgrids))
    up = oracle.inv2fwd_iso(k.xinv, k.yinv, k.zinv, gk, k.xgrids, k.ygrids, k.zgrids)
    assert np.array_equal(up, _py_inv2fwd(k.xinv, k.yinv, k.zinv, gk, k.xgrids, k.ygrids,
                                          k.zgrids))


def test_inv_grid_conserves_the_integral(oracle):
    """The trilinear weights of a node sum to one: each set's gk sums to the
    interior integral of adj (to rounding)."""
    k = W.kernel3d_case(nx=30, ny=24, nz=12, nperiod=1)
    rng = np.random.default_rng(5)
    adj = np.asfortranarray(rng.standard_normal((30, 24, 12)))
    gk = oracle.inv_grid_iso(k.xinv, k.yinv, k.zinv, adj, k.xgrids, k.ygrids, k.zgrids)
    dxyz = (k.xgrids[1] - k.xgrids[0]) * (k.ygrids[1] - k.ygrids[0]) * (k.zgrids[1] - k.zgrids[0])
    tot = adj[1:-1, 1:-1, 1:-1].sum() * dxyz
    ninv = k.xinv.shape[0] * k.yinv.shape[0] * k.zinv.shape[0]
    for s in range(k.xinv.shape[1]):
        assert abs(gk[s * ninv:(s + 1) * ninv].sum() / tot - 1) <= 1e-12


def test_inv2fwd_reproduces_linear_fields(oracle):
    """Trilinear interpolation is exact for a linear function of the node
    coordinates: update = nset * f(model node)."""
    k = W.kernel3d_case(nx=20, ny=16, nz=10, nperiod=1)
    f = lambda x, y, z: 0.3 + 1.7 * x - 0.4 * y + 0.05 * z
    nset = k.xinv.shape[1]
    gk = np.concatenate([f(k.xinv[:, s][:, None, None], k.yinv[:, s][None, :, None],
                           k.zinv[:, s][None, None, :]).ravel(order="F") for s in range(nset)])
    up = oracle.inv2fwd_iso(k.xinv, k.yinv, k.zinv, gk, k.xgrids, k.ygrids, k.zgrids)
    ref = nset * f(k.xgrids[:, None, None], k.ygrids[None, :, None], k.zgrids[None, None, :])
    assert rel_max(up, ref) <= 1e-12


def test_not_located_reports_first_node(oracle):
    vx, vy, vz, xinv, yinv, zinv = tie_grids(nset=1)
    xinv = xinv.copy(order="F")
    xinv[0, 0] = 0.5          # model x = 0 (only visited by inv2fwd_iso) is outside
    adj = np.zeros((7, 6, 5), order="F")
    oracle.inv_grid_iso(xinv, yinv, zinv, adj, vx, vy, vz)   # interior nodes: fine
    with pytest.raises(oracle.NotLocated) as e:
        oracle.inv2fwd_iso(xinv, yinv, zinv, np.zeros(4 * 4 * 4), vx, vy, vz)
    assert e.value.args[0] == (0.0, 0.0, 0.0)
    xinv[:, 0] = [1.5, 2.0, 3.0, 7.5]   # model x = 1 (interior) now outside too
    with pytest.raises(oracle.NotLocated) as e:
        oracle.inv_grid_iso(xinv, yinv, zinv, adj, vx, vy, vz)
    assert e.value.args[0] == (1.0, 1.0, 1.0)


def _py_dab(vs):
    c0, c1, c2, c3 = (float(F32(2.0947)), float(F32(2) * F32(0.8206)),
                      float(F32(3) * F32(0.2683)), float(F32(4) * F32(0.0251)))
    v2 = vs * vs
    return c0 - c1 * vs + c2 * v2 - c3 * (v2 * vs)


def _py_drda(vp):
    c0, c1, c2, c3, c4 = (float(F32(1.6612)), float(F32(2) * F32(0.4721)),
                          float(F32(3) * F32(0.0671)), float(F32(4) * F32(0.0043)),
                          float(F32(5) * F32(0.000106)))
    v2 = vp * vp
    return c0 - c1 * vp + c2 * v2 - c3 * (v2 * vp) + c4 * (v2 * v2)


@pytest.mark.parametrize("abr,rs", [(False, False), (True, False), (True, True)])
def test_combine_matches_element_restatement(oracle, abr, rs):
    k = W.kernel3d_case(nx=6, ny=5, nz=4, nperiod=3)
    ker, kd = oracle.combine_kernels(k.adj_s, k.adj_density, k.sen_vs, k.sen_vp, k.sen_rho,
                                     k.vs3d, k.vp3d, abr, rs)
    P, nx, ny, nz = k.sen_vs.shape
    rho = float(F32(0.33))
    for (x, y, z) in [(0, 0, 0), (5, 4, 3), (2, 3, 1), (4, 1, 2)]:
        kk = [0.0, 0.0, 0.0]
        dd = [0.0, 0.0, 0.0]
        dab, drda = _py_dab(float(k.vs3d[x, y, z])), _py_drda(float(k.vp3d[x, y, z]))
        for p in range(P):
            a, b = float(k.adj_s[p, x, y]), float(k.adj_density[p, x, y])
            s0, s1, s2 = (float(k.sen_vs[p, x, y, z]), float(k.sen_vp[p, x, y, z]),
                          float(k.sen_rho[p, x, y, z]))
            if abr:
                kk[0] = kk[0] - a * s0
                dd[0] = dd[0] - b * s0
                kk[1] = kk[1] - a * s1
                dd[1] = dd[1] - b * s1
                if not rs:
                    kk[2] = kk[2] - a * s2
                    dd[2] = dd[2] - b * s2
            else:
                kk[0] = kk[0] - a * s0 - a * s1 * dab - a * s2 * drda * dab
                dd[0] = dd[0] - b * s0 - b * s1 * dab - b * s2 * drda * dab
        if abr and rs:
            kk[2] = rho * kk[0]
            dd[2] = dd[0]
        n = 3 if abr else 1
        assert [ker[q, x, y, z] for q in range(n)] == kk[:n]
        assert [kd[q, x, y, z] for q in range(n)] == dd[:n]


def test_inv_grids_restatements_agree(oracle):
    xg, yg, zg = W.arange_grid(100.0, 60, 0.1), W.arange_grid(22.0, 60, 0.1), np.linspace(0, 60, 30)
    for ninv, nset in [((8, 9, 8), 5), ((8, 9, 10), 5), ((10, 11, 8), 3), ((6, 6, 5), 1)]:
        a = oracle.get_inv_grids(xg, yg, zg, ninv, nset)
        b = W.inv_grids(xg, yg, zg, ninv, nset)
        assert all(np.array_equal(u, v) for u, v in zip(a, b))


def test_post_process_preconditioning(oracle):
    """kdensity_coe > 0: ker scaled by 1/(|kd|/max|kd|)^coe where the ratio
    is >= 1e-4, zeroed below (regularize_ker_density)."""
    k = W.kernel3d_case(nx=12, ny=10, nz=6, nperiod=2)
    ker, kd = oracle.combine_kernels(k.adj_s, k.adj_density, k.sen_vs, k.sen_vp, k.sen_rho,
                                     k.vs3d, k.vp3d)
    kd = kd.copy(order="F")
    kd[0, 3, 3, 3] = 1e-9 * np.abs(kd).max()   # below the threshold
    ker2, grad = oracle.post_process_kernels(ker, kd, 1.0, k.xinv, k.yinv, k.zinv, k.xgrids,
                                             k.ygrids, k.zgrids, k.chi0, 0.5,
                                             np.zeros_like(ker))
    r = np.abs(kd[0]) / np.abs(kd[0]).max()
    exp = np.where(r < 1e-4, 0.0, ker[0] / r)
    assert ker2[0, 3, 3, 3] == 0.0
    assert rel_max(ker2[0], exp) <= 1e-15
    assert np.abs(grad).max() > 0
