"""ctypes wrapper of the CPU oracle (test infrastructure only).

The oracle is a plain-C restatement of the reference Fortran (see
``surfatt_oracle.c`` for the file:line map).  Only the test suite, the smoke
check and the benchmark's CPU-baseline leg import this module; the product
library never does.

Parity status: unpinned by the reference's own tests (it has none for this
path and cannot be built here); pinned by analytic known-answer,
reciprocity and finite-difference tests in ``tests/``.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libsurfatt_oracle.so")
# The same sources built -O3 with FP contraction on (the timed CPU baseline
# only; parity checks use the -ffp-contract=off build above).
_FAST_PATH = os.path.join(_HERE, "_build", "libsurfatt_oracle_fast.so")
FAST_FLAGS = "gcc -O3 (FP contraction: gcc default, FMA on aarch64)"
STRICT_FLAGS = "gcc -O2 -ffp-contract=off"
_lib = None
_fast = None

OK, SOURCE_ON_BOUNDARY, BAD_ARG, NOT_CONVERGED = 0, 1, 2, 3

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_llp = ctypes.POINTER(ctypes.c_longlong)


def build():
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.check_call(["make", "-s", "-C", _HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = ctypes.CDLL(_LIB_PATH)
        _lib.orc_gradient_eval_range.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp,
                                                 _ip, _ip, _ip]
        _lib.orc_post_process_kernels.argtypes = [ctypes.c_int] * 4 + [
            _dp, _dp, ctypes.c_double, _dp, _dp, _dp] + [ctypes.c_int] * 4 + [
            _dp, _dp, _dp, ctypes.c_double, ctypes.c_double, _dp, _dp]
    return _lib


def fast_lib():
    """The -O3 build of the same sources, for timing only."""
    global _fast
    if _fast is None:
        if not os.path.exists(_FAST_PATH):
            build()
        _fast = ctypes.CDLL(_FAST_PATH)
        _fast.orc_gradient_eval_range.argtypes = lib().orc_gradient_eval_range.argtypes
    return _fast


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _fortran2d(a):
    """(nx, ny) array -> column-major buffer (x fastest)."""
    return np.asfortranarray(a, dtype=np.float64)


def _solve(fn, xx, yy, a, b, c, fun, x0, y0):
    xx, yy = _f64(xx), _f64(yy)
    nx, ny = len(xx), len(yy)
    a, b, c, fun = (_fortran2d(v) for v in (a, b, c, fun))
    T = np.zeros((nx, ny), order="F")
    it = ctypes.c_int(0)
    st = fn(_d(xx), _d(yy), nx, ny, _d(a), _d(b), _d(c), _d(T), _d(fun), ctypes.c_double(x0),
            ctypes.c_double(y0), ctypes.byref(it))
    return T, st, it.value


def fsm_uw_ps_lonlat_2d(xx_deg, yy_deg, spha, sphb, sphc, fun, x0_deg, y0_deg):
    """Returns (T (nx, ny), status, iterations)."""
    return _solve(lib().orc_fsm_uw_ps_lonlat_2d, xx_deg, yy_deg, spha, sphb, sphc, fun, x0_deg,
                  y0_deg)


def fsm_uw_ps_cart_2d(xx, yy, a, b, c, fun, x0, y0):
    return _solve(lib().orc_fsm_uw_ps_cart_2d, xx, yy, a, b, c, fun, x0, y0)


def fsm_weno3_ps_multi_2d(xx, yy, a, b, c, fun, x0, y0):
    return _solve(lib().orc_fsm_weno3_ps_multi_2d, xx, yy, a, b, c, fun, x0, y0)


def fsm_weno3_ps_2d(xx, yy, a, b, c, fun, x0, y0):
    return _solve(lib().orc_fsm_weno3_ps_2d, xx, yy, a, b, c, fun, x0, y0)


def _adjoint(fn, xx, yy, a, b, c, T, xrec, yrec, sadj):
    xx, yy = _f64(xx), _f64(yy)
    nx, ny = len(xx), len(yy)
    a, b, c, T = (_fortran2d(v) for v in (a, b, c, T))
    xrec, yrec, sadj = _f64(xrec), _f64(yrec), _f64(sadj)
    Ta = np.zeros((nx, ny), order="F")
    it = ctypes.c_int(0)
    st = fn(_d(xx), _d(yy), nx, ny, _d(a), _d(b), _d(c), _d(T), _d(Ta), _d(xrec), _d(yrec),
            _d(sadj), len(xrec), ctypes.byref(it))
    return Ta, st, it.value


def fsm_o1_jse_lonlat_2d(xx_deg, yy_deg, spha, sphb, sphc, T, xrec_deg, yrec_deg, sadj):
    return _adjoint(lib().orc_fsm_o1_jse_lonlat_2d, xx_deg, yy_deg, spha, sphb, sphc, T,
                    xrec_deg, yrec_deg, sadj)


def fsm_o1_jse_2d(xx, yy, a, b, c, T, xrec, yrec, sadj):
    return _adjoint(lib().orc_fsm_o1_jse_2d, xx, yy, a, b, c, T, xrec, yrec, sadj)


def mask(xx, yy, table, x0, y0):
    xx, yy = _f64(xx), _f64(yy)
    t = _fortran2d(table).copy(order="F")
    lib().orc_mask(_d(xx), _d(yy), len(xx), len(yy), _d(t), ctypes.c_double(x0),
                   ctypes.c_double(y0))
    return t


def interp2(x, y, v, xq, yq):
    x, y = _f64(x), _f64(y)
    v = _fortran2d(v)
    out = ctypes.c_double(0)
    st = lib().orc_interp2(_d(x), len(x), _d(y), len(y), _d(v), ctypes.c_double(xq),
                           ctypes.c_double(yq), ctypes.byref(out))
    if st != OK:
        raise ValueError("interp2: query point outside the grid")
    return out.value


def gaussian_smooth_geo_2(data, lons, lats, sigma):
    """gaussian_smooth_geo_2 (src/shared/utils.f90:1194-1225) of one (nx, ny)
    field; lons / lats in degrees, sigma in degrees.  Returns (nx, ny)."""
    lons, lats = _f64(lons), _f64(lats)
    d = _fortran2d(data)
    nx, ny = d.shape
    out = np.zeros((nx, ny), order="F")
    lib().orc_gaussian_smooth_geo_2(_d(d), nx, ny, _d(lons), _d(lats), ctypes.c_double(sigma),
                                    _d(out))
    return out


class _Problem(ctypes.Structure):
    _fields_ = [("nperiod", ctypes.c_int), ("nx", _ip), ("ny", _ip), ("xoff", _llp),
                ("yoff", _llp), ("goff", _llp), ("xgrid", _dp), ("ygrid", _dp),
                ("svel", _dp), ("m11", _dp), ("m12", _dp), ("m22", _dp),
                ("nsolve", ctypes.c_int), ("pidx", _ip), ("srcx", _dp), ("srcy", _dp),
                ("rec_off", _ip), ("nrec", _ip), ("recx", _dp), ("recy", _dp), ("tt", _dp),
                ("weight", _dp), ("path", _ip), ("npath", ctypes.c_int)]


def gradient_eval(pb, mode=2, nthreads=1, s_begin=0, s_end=None, timed=False):
    """One gradient evaluation of a packed problem (see surfatt_gb300.workloads.Problem).

    mode 0: forward only; 2: tomo2d (adj/svel^2); 3: 3-D (adj and density /svel^3).
    timed: run the -O3 build (the CPU baseline's timing) instead of the
    parity build.
    Returns dict(adj_s, adj_density, chi, tt_fwd, status, fwd_iters, adj_iters, rc).
    """
    if s_end is None:
        s_end = pb.nsolve
    keep = []

    def P(a, kind):
        a = np.ascontiguousarray(a, dtype={"d": np.float64, "i": np.int32, "q": np.int64}[kind])
        keep.append(a)
        return a.ctypes.data_as({"d": _dp, "i": _ip, "q": _llp}[kind])

    s = _Problem(pb.nperiod, P(pb.nx, "i"), P(pb.ny, "i"), P(pb.xoff, "q"), P(pb.yoff, "q"),
                 P(pb.goff, "q"), P(pb.xgrid, "d"), P(pb.ygrid, "d"), P(pb.svel, "d"),
                 P(pb.m11, "d"), P(pb.m12, "d"), P(pb.m22, "d"), pb.nsolve, P(pb.pidx, "i"),
                 P(pb.srcx, "d"), P(pb.srcy, "d"), P(pb.rec_off, "i"), P(pb.nrec, "i"),
                 P(pb.recx, "d"), P(pb.recy, "d"), P(pb.tt, "d"), P(pb.weight, "d"),
                 P(pb.path, "i"), pb.npath)
    ncell = pb.ncell
    adj_s = np.zeros(ncell)
    adj_d = np.zeros(ncell)
    chi = ctypes.c_double(0)
    tt_fwd = np.zeros(max(pb.npath, 1))
    status = np.zeros(pb.nsolve, np.int32)
    fit = np.zeros(pb.nsolve, np.int32)
    ait = np.zeros(pb.nsolve, np.int32)
    rc = (fast_lib() if timed else lib()).orc_gradient_eval_range(
        ctypes.byref(s), mode, nthreads, s_begin, s_end,
                                       _d(adj_s), _d(adj_d), ctypes.byref(chi), _d(tt_fwd),
                                       _i(status), _i(fit), _i(ait))
    return dict(adj_s=adj_s, adj_density=adj_d, chi=chi.value, tt_fwd=tt_fwd[:pb.npath],
                status=status, fwd_iters=fit, adj_iters=ait, rc=rc)


def scatter_all_i(countval, size, rank):
    a, b = ctypes.c_int(0), ctypes.c_int(0)
    lib().orc_scatter_all_i(countval, size, rank, ctypes.byref(a), ctypes.byref(b))
    return a.value, b.value


# ---------------------------------------------------------------------------
# Kernel combination and multigrid projection (oracle_project.c)
# ---------------------------------------------------------------------------
def _F(a):
    return np.asfortranarray(a, dtype=np.float64)


def combine_kernels(adj_s, adj_density, sen_vs, sen_vp, sen_rho, vs3d, vp3d,
                    use_alpha_beta_rho=False, rho_scaling=False):
    """combine_kernels (src/acqui.f90:196-245).  adj_s (P, nx, ny), sen_*
    (P, nx, ny, nz), vs3d / vp3d (nx, ny, nz), Fortran order.  Returns
    (ker, ker_density), each (nker, nx, ny, nz)."""
    adj_s, adj_density = _F(adj_s), _F(adj_density)
    sen_vs, sen_vp, sen_rho = _F(sen_vs), _F(sen_vp), _F(sen_rho)
    vs3d, vp3d = _F(vs3d), _F(vp3d)
    P, nx, ny, nz = sen_vs.shape
    nker = 3 if use_alpha_beta_rho else 1
    ker = np.zeros((nker, nx, ny, nz), order="F")
    kd = np.zeros((nker, nx, ny, nz), order="F")
    lib().orc_combine_kernels(P, nx, ny, nz, _d(adj_s), _d(adj_density), _d(sen_vs), _d(sen_vp),
                              _d(sen_rho), _d(vs3d), _d(vp3d), int(bool(use_alpha_beta_rho)),
                              int(bool(rho_scaling)), _d(ker), _d(kd))
    return ker, kd


def dalpha_dbeta(vs):
    return lib_f("orc_dalpha_dbeta_1")(float(vs))


def drho_dalpha(vp):
    return lib_f("orc_drho_dalpha_1")(float(vp))


def lib_f(name):
    f = getattr(lib(), name)
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_double]
    return f


class NotLocated(RuntimeError):
    """A model node lies outside the inversion grids (the reference stops)."""


def inv_grid_iso(xinv, yinv, zinv, adj, vel_x, vel_y, vel_z):
    """inv_grid_iso (src/eikon_solver_2d.f90:1541-1614).  xinv (nxinv, nset)
    ..., adj (nx, ny, nz).  Returns gk (nset * nxinv * nyinv * nzinv)."""
    xinv, yinv, zinv, adj = _F(xinv), _F(yinv), _F(zinv), _F(adj)
    nx, ny, nz = adj.shape
    nset = xinv.shape[1]
    gk = np.zeros(nset * xinv.shape[0] * yinv.shape[0] * zinv.shape[0])
    bad = np.zeros(3)
    rc = lib().orc_inv_grid_iso(_d(xinv), _d(yinv), _d(zinv), xinv.shape[0], yinv.shape[0],
                                zinv.shape[0], nset, _d(adj), nx, ny, nz, _d(gk),
                                _d(_f64(vel_x)), _d(_f64(vel_y)), _d(_f64(vel_z)), _d(bad))
    if rc:
        raise NotLocated(tuple(bad))
    return gk


def inv2fwd_iso(xinv, yinv, zinv, gk, vel_x, vel_y, vel_z):
    """inv2fwd_iso (src/eikon_solver_2d.f90:1617-1691).  Returns update
    (nx, ny, nz), Fortran order."""
    xinv, yinv, zinv = _F(xinv), _F(yinv), _F(zinv)
    vel_x, vel_y, vel_z = _f64(vel_x), _f64(vel_y), _f64(vel_z)
    nx, ny, nz = len(vel_x), len(vel_y), len(vel_z)
    upd = np.zeros((nx, ny, nz), order="F")
    bad = np.zeros(3)
    rc = lib().orc_inv2fwd_iso(_d(xinv), _d(yinv), _d(zinv), xinv.shape[0], yinv.shape[0],
                               zinv.shape[0], xinv.shape[1], nx, ny, nz, _d(_f64(gk)), _d(vel_x),
                               _d(vel_y), _d(vel_z), _d(upd), _d(bad))
    if rc:
        raise NotLocated(tuple(bad))
    return upd


def post_process_kernels(ker, ker_density, kdensity_coe, xinv, yinv, zinv, xgrids, ygrids,
                         zgrids, chi0, weight, gradient_s):
    """post_processing_for_kernel (src/acqui.f90:247-286).  ker / ker_density
    / gradient_s (nker, nx, ny, nz).  Returns (ker after preconditioning,
    gradient_s after accumulation) as new arrays."""
    ker = _F(ker).copy(order="F")
    kd = _F(ker_density)
    grad = _F(gradient_s).copy(order="F")
    xinv, yinv, zinv = _F(xinv), _F(yinv), _F(zinv)
    nker, nx, ny, nz = ker.shape
    bad = np.zeros(3)
    rc = lib().orc_post_process_kernels(
        nker, nx, ny, nz, _d(ker), _d(kd), ctypes.c_double(kdensity_coe), _d(xinv), _d(yinv),
        _d(zinv), xinv.shape[0], yinv.shape[0], zinv.shape[0], xinv.shape[1],
        _d(_f64(xgrids)), _d(_f64(ygrids)), _d(_f64(zgrids)), ctypes.c_double(chi0),
        ctypes.c_double(weight), _d(grad), _d(bad))
    if rc:
        raise NotLocated(tuple(bad))
    return ker, grad


def get_inv_grids(xgrids, ygrids, zgrids, n_inv_grid, nset):
    """get_inv_grids (src/model.f90:127-172): (xinv, yinv, zinv), each
    (ninv, nset) Fortran order."""
    xg, yg, zg = _f64(xgrids), _f64(ygrids), _f64(zgrids)
    nix, niy, niz = (int(v) for v in n_inv_grid)
    xinv = np.zeros((nix, nset), order="F")
    yinv = np.zeros((niy, nset), order="F")
    zinv = np.zeros((niz, nset), order="F")
    lib().orc_get_inv_grids(_d(xg), len(xg), _d(yg), len(yg), _d(zg), len(zg), nix, niy, niz,
                            nset, _d(xinv), _d(yinv), _d(zinv))
    return xinv, yinv, zinv


# ---------------------------------------------------------------------------
# Work list and receiver gathers from a src_rec table (oracle_srcrec.c)
# ---------------------------------------------------------------------------
def srcrec_worklist(evtname, staname, stla, stlo, evla, evlo, period, tt, weight=None):
    """scatter_src_gather + get_recs over a src_rec table (lists of names,
    arrays of values).  Returns a dict: periods, station names / lon / lat,
    and per solve pidx, sta, srcx, srcy, rec_off, nrec; per receiver recx,
    recy, tt, weight, path (0-based)."""
    n = len(tt)
    enc = lambda names: (ctypes.c_char_p * n)(*[str(v).encode() for v in names])
    ev, st = enc(evtname), enc(staname)
    f = lambda a: _f64(a)
    stla, stlo, evla, evlo, period, tt = (f(a) for a in (stla, stlo, evla, evlo, period, tt))
    w = None if weight is None else f(weight)
    npr, nst, nso = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
    periods = np.zeros(n)
    sname = (ctypes.c_char_p * (2 * n))()
    slo, sla = np.zeros(2 * n), np.zeros(2 * n)
    ints = {k: np.zeros(n, np.int32) for k in ("pidx", "sta", "rec_off", "nrec", "path")}
    dbl = {k: np.zeros(n) for k in ("srcx", "srcy", "recx", "recy", "tt", "weight")}
    rc = lib().orc_srcrec_worklist(
        n, ev, st, _d(stla), _d(stlo), _d(evla), _d(evlo), _d(period), _d(tt),
        _d(w) if w is not None else None, ctypes.byref(npr), _d(periods), ctypes.byref(nst),
        sname, _d(slo), _d(sla), ctypes.byref(nso), _i(ints["pidx"]), _i(ints["sta"]),
        _d(dbl["srcx"]), _d(dbl["srcy"]), _i(ints["rec_off"]), _i(ints["nrec"]),
        _d(dbl["recx"]), _d(dbl["recy"]), _d(dbl["tt"]), _d(dbl["weight"]), _i(ints["path"]))
    if rc:
        raise ValueError("srcrec_worklist: bad table")
    P, S, NS = npr.value, nst.value, nso.value
    out = dict(periods=periods[:P], sta_name=[sname[i].decode() for i in range(S)],
               sta_lo=slo[:S], sta_la=sla[:S])
    for k in ("pidx", "sta", "rec_off", "nrec"):
        out[k] = ints[k][:NS]
    for k in ("srcx", "srcy"):
        out[k] = dbl[k][:NS]
    for k in ("recx", "recy", "tt", "weight"):
        out[k] = dbl[k][:n]
    out["path"] = ints["path"][:n]
    return out


# ---------------------------------------------------------------------------
# Surface metric from topography (oracle_topo.c)
# ---------------------------------------------------------------------------
def gradient_2_geo(f, lon, lat):
    """gradient_2_geo (src/shared/utils.f90:1118-1160): (tx, ty), (nx, ny)."""
    f = _fortran2d(f)
    nx, ny = f.shape
    tx = np.zeros((nx, ny), order="F")
    ty = np.zeros((nx, ny), order="F")
    lib().orc_gradient_2_geo(_d(f), nx, ny, _d(_f64(lon)), _d(_f64(lat)), _d(tx), _d(ty))
    return tx, ty


def topo_metric(topo, lon, lat, sigma):
    """get_topo's per-period loop (src/grid.f90:117-145): topo (nx, ny) in
    km, one sigma (degrees) per period.  Returns (m11, m22, m12, angle), each
    (nperiod, nx, ny) in Fortran order, as grid.f90 stores them."""
    topo = _fortran2d(topo)
    nx, ny = topo.shape
    sigma = _f64(np.atleast_1d(sigma))
    P = len(sigma)
    outs = [np.zeros((P, nx, ny), order="F") for _ in range(4)]
    rc = lib().orc_topo_metric(_d(topo), nx, ny, _d(_f64(lon)), _d(_f64(lat)), P, _d(sigma),
                               *[_d(o) for o in outs])
    if rc:
        raise ValueError("topo_metric: bad grid")
    return tuple(outs)
