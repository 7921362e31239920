"""Python host binding of libsurfatt_gb300.so (SurfATT travel-time + adjoint
path on GB300).

This module is a thin ctypes layer over the C ABI declared in
``include/surfatt_gb300.h``; every computation runs in the CUDA library.
There is no CPU fallback: if the library is missing or no GPU is present the
calls raise.

Names follow the reference:
  * ``fsm_uw_ps_lonlat_2d`` / ``fsm_o1_jse_lonlat_2d`` / ``mask`` ... call the
    drop-in symbols that replace the routines of src/eikon_solver_2d.f90;
  * ``MeasAdj`` mirrors ``att_measadj`` (src/measadj.f90:25-114);
  * ``Engine`` runs whole gradient evaluations (the per-(period, source) loop
    of src/acqui.f90:91-161 / src/tomo2d.f90:158-201 with the kernel sums).
"""
import ctypes
import os

import numpy as np

from . import _build
from .workloads import Problem  # noqa: F401

OK, SOURCE_ON_BOUNDARY, BAD_ARG, NOT_CONVERGED, OOM, CUDA_ERROR, TIMEOUT = range(7)
STATUS_NAMES = {0: "OK", 1: "SOURCE_ON_BOUNDARY", 2: "BAD_ARG", 3: "NOT_CONVERGED", 4: "OOM",
                5: "CUDA_ERROR", 6: "TIMEOUT"}
PREC_FP64, PREC_FP32 = 0, 1
MODE_FORWARD, MODE_2D, MODE_3D = 0, 2, 3

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_llp = ctypes.POINTER(ctypes.c_longlong)
_lib = None

# every symbol the header declares (checked by the CPU test suite)
EXPORTED = [
    "fsm_uw_ps_lonlat_2d_", "fsm_uw_ps_cart_2d_", "fsm_weno3_ps_2d_", "fsm_weno3_ps_multi_2d_",
    "fsm_o1_jse_lonlat_2d_", "fsm_o1_jse_2d_", "mask_", "surfatt_last_status",
    "surfatt_last_iterations", "surfatt_set_exit_on_boundary", "surfatt_measadj_run_forward",
    "surfatt_measadj_run_adjoint", "surfatt_measadj_run_adjoint_density",
    "surfatt_engine_create", "surfatt_engine_destroy", "surfatt_engine_load",
    "surfatt_engine_update_velocity", "surfatt_engine_run", "surfatt_engine_sync",
    "surfatt_engine_results", "surfatt_engine_timing", "surfatt_engine_work", "surfatt_version",
    "surfatt_engine_launch_config", "surfatt_engine_autotune", "surfatt_engine_kernel_variant",
    "surfatt_engine_set_graphs", "surfatt_engine_set_kernel", "surfatt_engine_set_profile",
    "surfatt_engine_phase_cycles", "surfatt_gaussian_smooth_geo_2", "surfatt_engine_smooth",
    "surfatt_engine_smooth_timing", "inv_grid_iso_", "inv2fwd_iso_", "surfatt_combine_kernels",
    "surfatt_post_process_kernels", "surfatt_kernel_gradient", "surfatt_kernel_gradient_timing",
    "surfatt_srcrec_read_csv", "surfatt_srcrec_create", "surfatt_srcrec_destroy",
    "surfatt_srcrec_info", "surfatt_srcrec_periods", "surfatt_srcrec_stations",
    "surfatt_srcrec_station_name", "surfatt_srcrec_paths", "surfatt_srcrec_build_worklist",
    "surfatt_srcrec_worklist", "surfatt_srcrec_build_timing", "surfatt_srcrec_write_csv",
    "surfatt_topo_metric", "surfatt_topo_sigma", "surfatt_topo_metric_timing",
    "surfatt_measure_peaks", "surfatt_uw_lonlat_solve_noalloc", "surfatt_engine_device_results",
    "surfatt_engine_set_keep_fields", "surfatt_engine_fields", "surfatt_engine_test_hold",
    "surfatt_server_create", "surfatt_server_destroy", "surfatt_server_add_model",
    "surfatt_server_add_worklist", "surfatt_server_submit", "surfatt_server_wait",
    "surfatt_server_stats", "surfatt_server_reset_stats",
]


class SurfattError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        super().__init__(f"{what}: {STATUS_NAMES.get(status, status)}")


def build(force=False, verbose=False):
    """Compile libsurfatt_gb300.so for sm_103a (in-tree)."""
    return _build.build(force=force, verbose=verbose)


def library_path():
    return _build.LIB_PATH


def lib():
    """Load the CUDA library (it must have been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_build.LIB_PATH):
            raise RuntimeError("libsurfatt_gb300.so is not built: run surfatt_gb300.build() "
                               "(the library is the only implementation; there is no fallback)")
        L = ctypes.CDLL(_build.LIB_PATH)
        L.surfatt_version.restype = ctypes.c_char_p
        L.surfatt_engine_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                            ctypes.c_size_t]
        for f in ("surfatt_engine_destroy",):
            getattr(L, f).argtypes = [ctypes.c_void_p]
            getattr(L, f).restype = None
        L.surfatt_engine_load.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.surfatt_engine_update_velocity.argtypes = [ctypes.c_void_p, _dp]
        L.surfatt_engine_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.surfatt_engine_sync.argtypes = [ctypes.c_void_p]
        L.surfatt_engine_results.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.surfatt_engine_timing.argtypes = [ctypes.c_void_p, _dp, _dp, _ip]
        L.surfatt_engine_work.argtypes = [ctypes.c_void_p, _dp, _dp]
        dd = ctypes.c_double
        L.surfatt_measadj_run_forward.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_int, _dp, _dp,
                                                  _dp, _dp, dd, dd, ctypes.c_int, _dp, _dp, _dp,
                                                  _dp, _dp, _dp, _dp]
        L.surfatt_measadj_run_adjoint.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_int, _dp, _dp,
                                                  _dp, dd, dd, ctypes.c_int, _dp, _dp, _dp, _dp,
                                                  _dp, _dp, _dp]
        L.surfatt_measadj_run_adjoint_density.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_int,
                                                          _dp, _dp, _dp, dd, dd, ctypes.c_int,
                                                          _dp, _dp, _dp, _dp, _dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _f2(a):
    return np.asfortranarray(a, dtype=np.float64)


def measure_peaks(device=0):
    """(fp64_tflops, fp32_tflops) FMA issue peaks measured on `device`."""
    a, b = ctypes.c_double(0), ctypes.c_double(0)
    st = lib().surfatt_measure_peaks(int(device), ctypes.byref(a), ctypes.byref(b))
    if st != OK:
        raise SurfattError(st, "measure_peaks")
    return a.value, b.value


def uw_lonlat_solve_noalloc(xx_deg, yy_deg, nx, ny, spha, sphb, sphc, fun, x0_deg, y0_deg, T,
                            status_iters, stream=0):
    """surfatt_uw_lonlat_solve_noalloc on device pointers (integers), e.g.
    torch tensors' data_ptr(); enqueued on `stream`, returns the launch status.
    For callers that must not allocate device memory at call time; the
    library's fixed scratch limits grids to 16384 cells."""
    L = lib()
    f = L.surfatt_uw_lonlat_solve_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                  ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f(xx_deg, yy_deg, int(nx), int(ny), spha, sphb, sphc, fun, float(x0_deg),
             float(y0_deg), T, status_iters, stream)


def last_status():
    return lib().surfatt_last_status()


def last_iterations():
    return lib().surfatt_last_iterations()


def set_exit_on_boundary(enable: bool):
    lib().surfatt_set_exit_on_boundary(int(bool(enable)))


# ---------------------------------------------------------------------------
# drop-in symbols (called exactly as gfortran would: every argument by reference)
# ---------------------------------------------------------------------------
def _ci(v):
    return ctypes.byref(ctypes.c_int(int(v)))


def _cd(v):
    return ctypes.byref(ctypes.c_double(float(v)))


def _fwd_call(name, xx, yy, a, b, c, fun, x0, y0):
    xx, yy = _c64(xx), _c64(yy)
    nx, ny = len(xx), len(yy)
    a, b, c, fun = (_f2(v) for v in (a, b, c, fun))
    T = np.zeros((nx, ny), order="F")
    u = np.zeros((nx, ny), order="F")
    getattr(lib(), name)(_d(xx), _d(yy), _ci(nx), _ci(ny), _d(a), _d(b), _d(c), _d(T), _d(fun),
                         _cd(x0), _cd(y0), _d(u))
    return T, last_status(), last_iterations()


def fsm_uw_ps_lonlat_2d(xx_deg, yy_deg, spha, sphb, sphc, fun, x0_deg, y0_deg):
    """FSM_UW_PS_lonlat_2d on the GPU; returns (T (nx, ny), status, iterations)."""
    return _fwd_call("fsm_uw_ps_lonlat_2d_", xx_deg, yy_deg, spha, sphb, sphc, fun, x0_deg, y0_deg)


def fsm_uw_ps_cart_2d(xx, yy, a, b, c, fun, x0, y0):
    return _fwd_call("fsm_uw_ps_cart_2d_", xx, yy, a, b, c, fun, x0, y0)


def fsm_weno3_ps_2d(xx, yy, a, b, c, fun, x0, y0):
    return _fwd_call("fsm_weno3_ps_2d_", xx, yy, a, b, c, fun, x0, y0)


def fsm_weno3_ps_multi_2d(xx, yy, a, b, c, fun, x0, y0):
    return _fwd_call("fsm_weno3_ps_multi_2d_", xx, yy, a, b, c, fun, x0, y0)


def _adj_call(name, xx, yy, a, b, c, T, xrec, yrec, sadj):
    xx, yy = _c64(xx), _c64(yy)
    nx, ny = len(xx), len(yy)
    a, b, c, T = (_f2(v) for v in (a, b, c, T))
    xrec, yrec, sadj = _c64(xrec), _c64(yrec), _c64(sadj)
    Ta = np.zeros((nx, ny), order="F")
    getattr(lib(), name)(_d(xx), _d(yy), _ci(nx), _ci(ny), _d(a), _d(b), _d(c), _d(T), _d(Ta),
                         _d(xrec), _d(yrec), _d(sadj), _ci(len(xrec)))
    return Ta, last_status(), last_iterations()


def fsm_o1_jse_lonlat_2d(xx_deg, yy_deg, spha, sphb, sphc, T, xrec_deg, yrec_deg, sadj):
    return _adj_call("fsm_o1_jse_lonlat_2d_", xx_deg, yy_deg, spha, sphb, sphc, T, xrec_deg,
                     yrec_deg, sadj)


def fsm_o1_jse_2d(xx, yy, a, b, c, T, xrec, yrec, sadj):
    return _adj_call("fsm_o1_jse_2d_", xx, yy, a, b, c, T, xrec, yrec, sadj)


def mask(xx, yy, table, x0, y0):
    xx, yy = _c64(xx), _c64(yy)
    t = _f2(table).copy(order="F")
    lib().mask_(_d(xx), _d(yy), _ci(len(xx)), _ci(len(yy)), _d(t), _cd(x0), _cd(y0))
    st = last_status()
    if st != OK:
        raise SurfattError(st, "mask")
    return t


def gaussian_smooth_geo_2(data, lons, lats, sigma):
    """gaussian_smooth_geo_2 (src/shared/utils.f90:1194-1225): great-circle
    Gaussian smoothing of an (nx, ny) field on the lon/lat grid lons x lats
    (degrees, uniform), sigma in degrees.  Returns the smoothed (nx, ny)
    field (Fortran order)."""
    lons, lats = _c64(lons), _c64(lats)
    d = _f2(data)
    nx, ny = d.shape
    if len(lons) != nx or len(lats) != ny:
        raise ValueError("gaussian_smooth_geo_2: axes do not match the field")
    out = np.zeros((nx, ny), order="F")
    L = lib()
    L.surfatt_gaussian_smooth_geo_2.argtypes = [_dp, ctypes.c_int, ctypes.c_int, _dp, _dp,
                                                ctypes.c_double, _dp]
    st = L.surfatt_gaussian_smooth_geo_2(_d(d), nx, ny, _d(lons), _d(lats), float(sigma),
                                         _d(out))
    if st != OK:
        raise SurfattError(st, "gaussian_smooth_geo_2")
    return out


# ---------------------------------------------------------------------------
# Kernel combination and multigrid projection (3-D inversion)
# ---------------------------------------------------------------------------
def _F(a):
    return np.asfortranarray(a, dtype=np.float64)


def inv_grid_iso(xinv, yinv, zinv, adj, vel_x, vel_y, vel_z):
    """inv_grid_iso (src/eikon_solver_2d.f90:1541-1614) through the drop-in
    symbol: xinv (nxinv, nset), ..., adj (nx, ny, nz).  Returns gk
    (nset*nxinv*nyinv*nzinv).  A model node outside the inversion grids ends
    the process as the reference's `stop` does, unless
    set_exit_on_boundary(False), when SurfattError(BAD_ARG) is raised."""
    xinv, yinv, zinv, adj = _F(xinv), _F(yinv), _F(zinv), _F(adj)
    vx, vy, vz = _c64(vel_x), _c64(vel_y), _c64(vel_z)
    nx, ny, nz = adj.shape
    gk = np.zeros(xinv.shape[1] * xinv.shape[0] * yinv.shape[0] * zinv.shape[0])
    lib().inv_grid_iso_(_d(xinv), _d(yinv), _d(zinv), _ci(xinv.shape[0]), _ci(yinv.shape[0]),
                        _ci(zinv.shape[0]), _ci(xinv.shape[1]), _d(adj), _ci(nx), _ci(ny),
                        _ci(nz), _d(gk), _d(vx), _d(vy), _d(vz))
    st = last_status()
    if st != OK:
        raise SurfattError(st, "inv_grid_iso")
    return gk


def inv2fwd_iso(xinv, yinv, zinv, gk, vel_x, vel_y, vel_z):
    """inv2fwd_iso (src/eikon_solver_2d.f90:1617-1691) through the drop-in
    symbol.  Returns update (nx, ny, nz), Fortran order."""
    xinv, yinv, zinv = _F(xinv), _F(yinv), _F(zinv)
    vx, vy, vz = _c64(vel_x), _c64(vel_y), _c64(vel_z)
    gk = _c64(gk)
    upd = np.zeros((len(vx), len(vy), len(vz)), order="F")
    lib().inv2fwd_iso_(_d(xinv), _d(yinv), _d(zinv), _ci(xinv.shape[0]), _ci(yinv.shape[0]),
                       _ci(zinv.shape[0]), _ci(xinv.shape[1]), _ci(len(vx)), _ci(len(vy)),
                       _ci(len(vz)), _d(gk), _d(vx), _d(vy), _d(vz), _d(upd))
    st = last_status()
    if st != OK:
        raise SurfattError(st, "inv2fwd_iso")
    return upd


def combine_kernels(adj_s, adj_density, sen_vs, sen_vp, sen_rho, vs3d=None, vp3d=None,
                    use_alpha_beta_rho=False, rho_scaling=False):
    """combine_kernels (src/acqui.f90:196-245): adj_s / adj_density
    (P, nx, ny), sen_* (P, nx, ny, nz), vs3d / vp3d (nx, ny, nz).  Returns
    (ker, ker_density), (nker, nx, ny, nz) Fortran order."""
    adj_s, adj_density = _F(adj_s), _F(adj_density)
    sen_vs, sen_vp, sen_rho = _F(sen_vs), _F(sen_vp), _F(sen_rho)
    P, nx, ny, nz = sen_vs.shape
    vs3d = _F(vs3d) if vs3d is not None else np.zeros((nx, ny, nz), order="F")
    vp3d = _F(vp3d) if vp3d is not None else np.zeros((nx, ny, nz), order="F")
    nker = 3 if use_alpha_beta_rho else 1
    ker = np.zeros((nker, nx, ny, nz), order="F")
    kd = np.zeros((nker, nx, ny, nz), order="F")
    L = lib()
    L.surfatt_combine_kernels.argtypes = [ctypes.c_int] * 4 + [_dp] * 7 + [ctypes.c_int] * 2 + \
        [_dp] * 2
    st = L.surfatt_combine_kernels(P, nx, ny, nz, _d(adj_s), _d(adj_density), _d(sen_vs),
                                   _d(sen_vp), _d(sen_rho), _d(vs3d), _d(vp3d),
                                   int(bool(use_alpha_beta_rho)), int(bool(rho_scaling)), _d(ker),
                                   _d(kd))
    if st != OK:
        raise SurfattError(st, "combine_kernels")
    return ker, kd


def post_process_kernels(ker, ker_density, kdensity_coe, xinv, yinv, zinv, xgrids, ygrids,
                         zgrids, chi0, weight, gradient_s):
    """post_processing_for_kernel (src/acqui.f90:247-286).  Returns (ker
    after preconditioning, gradient_s + the kernels' update), new arrays."""
    ker = _F(ker).copy(order="F")
    kd = _F(ker_density)
    grad = _F(gradient_s).copy(order="F")
    xinv, yinv, zinv = _F(xinv), _F(yinv), _F(zinv)
    nker, nx, ny, nz = ker.shape
    L = lib()
    L.surfatt_post_process_kernels.argtypes = [ctypes.c_int] * 4 + [_dp, _dp, ctypes.c_double,
                                                                      _dp, _dp, _dp] + \
        [ctypes.c_int] * 4 + [_dp, _dp, _dp, ctypes.c_double, ctypes.c_double, _dp]
    st = L.surfatt_post_process_kernels(nker, nx, ny, nz, _d(ker), _d(kd), float(kdensity_coe),
                                        _d(xinv), _d(yinv), _d(zinv), xinv.shape[0],
                                        yinv.shape[0], zinv.shape[0], xinv.shape[1],
                                        _d(_c64(xgrids)), _d(_c64(ygrids)), _d(_c64(zgrids)),
                                        float(chi0), float(weight), _d(grad))
    if st != OK:
        raise SurfattError(st, "post_process_kernels")
    return ker, grad


def kernel_gradient(k, use_alpha_beta_rho=False, rho_scaling=False, kdensity_coe=0.0,
                    gradient_s=None, out=None):
    """combine_kernels + post_processing_for_kernel in one call (kernels
    stay on the device) for a workloads.Kernel3D `k`.  Returns (ker,
    ker_density, gradient_s).  `out`: optional dict of preallocated
    Fortran-order arrays ker / ker_density / gradient_s (e.g. pinned)."""
    P, nx, ny, nz = k.sen_vs.shape
    nker = 3 if use_alpha_beta_rho else 1
    if out is None:
        out = {n: np.zeros((nker, nx, ny, nz), order="F")
               for n in ("ker", "ker_density", "gradient_s")}
        if gradient_s is not None:
            out["gradient_s"][...] = gradient_s
    L = lib()
    L.surfatt_kernel_gradient.argtypes = [ctypes.c_int] * 4 + [_dp] * 7 + [ctypes.c_int] * 2 + \
        [ctypes.c_double] + [_dp] * 3 + [ctypes.c_int] * 4 + [_dp] * 3 + [ctypes.c_double] * 2 + \
        [_dp] * 3
    st = L.surfatt_kernel_gradient(
        P, nx, ny, nz, _d(k.adj_s), _d(k.adj_density), _d(k.sen_vs), _d(k.sen_vp),
        _d(k.sen_rho), _d(k.vs3d), _d(k.vp3d), int(bool(use_alpha_beta_rho)),
        int(bool(rho_scaling)), float(kdensity_coe), _d(k.xinv), _d(k.yinv), _d(k.zinv),
        k.xinv.shape[0], k.yinv.shape[0], k.zinv.shape[0], k.xinv.shape[1], _d(k.xgrids),
        _d(k.ygrids), _d(k.zgrids), float(k.chi0), float(k.weight), _d(out["ker"]),
        _d(out["ker_density"]), _d(out["gradient_s"]))
    if st != OK:
        raise SurfattError(st, "kernel_gradient")
    return out["ker"], out["ker_density"], out["gradient_s"]


def kernel_gradient_timing():
    """(device ms, kernel launches) of this thread's last combine /
    post-process / kernel-gradient call."""
    L = lib()
    L.surfatt_kernel_gradient_timing.argtypes = [_dp, _ip]
    ms, n = ctypes.c_double(0), ctypes.c_int(0)
    st = L.surfatt_kernel_gradient_timing(ctypes.byref(ms), ctypes.byref(n))
    if st != OK:
        raise SurfattError(st, "kernel_gradient_timing")
    return ms.value, n.value


# ---------------------------------------------------------------------------
# Surface metric from topography
# ---------------------------------------------------------------------------
def topo_metric(topo, lon, lat, sigma, angle=True):
    """get_topo's per-period loop (src/grid.f90:117-145) on the GPU: topo
    (nx, ny) km, one sigma (degrees) per period.  Returns (m11, m22, m12,
    topo_angle), each (nperiod, nx, ny) Fortran order (angle None when not
    asked for)."""
    topo = _f2(topo)
    nx, ny = topo.shape
    sigma = _c64(np.atleast_1d(sigma))
    P = len(sigma)
    outs = [np.zeros((P, nx, ny), order="F") for _ in range(3)]
    ang = np.zeros((P, nx, ny), order="F") if angle else None
    L = lib()
    L.surfatt_topo_metric.argtypes = [_dp, ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_int,
                                      _dp, _dp, _dp, _dp, _dp]
    st = L.surfatt_topo_metric(_d(topo), nx, ny, _d(_c64(lon)), _d(_c64(lat)), P, _d(sigma),
                               *[_d(o) for o in outs], _d(ang) if angle else None)
    if st != OK:
        raise SurfattError(st, "topo_metric")
    return outs[0], outs[1], outs[2], ang


def topo_sigma(phase_vel, periods, wavelen_factor):
    """sigma per period of src/grid.f90:117."""
    v, T = _c64(phase_vel), _c64(periods)
    out = np.zeros(len(v))
    L = lib()
    L.surfatt_topo_sigma.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_double, _dp]
    st = L.surfatt_topo_sigma(len(v), _d(v), _d(T), float(wavelen_factor), _d(out))
    if st != OK:
        raise SurfattError(st, "topo_sigma")
    return out


def topo_metric_timing():
    L = lib()
    L.surfatt_topo_metric_timing.argtypes = [_dp, _ip]
    ms, n = ctypes.c_double(0), ctypes.c_int(0)
    st = L.surfatt_topo_metric_timing(ctypes.byref(ms), ctypes.byref(n))
    if st != OK:
        raise SurfattError(st, "topo_metric_timing")
    return ms.value, n.value


# ---------------------------------------------------------------------------
# The src_rec table and its work list
# ---------------------------------------------------------------------------
class SrcRec:
    """A src_rec table (src/shared/src_rec_parser.f90, src/src_rec.f90):
    read_csv / from_arrays, the period and station tables, the GPU-built
    work list (scatter_src_gather + get_evt_gather) and write_csv."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def read_csv(cls, fname):
        h = ctypes.c_void_p()
        L = lib()
        L.surfatt_srcrec_read_csv.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]
        st = L.surfatt_srcrec_read_csv(str(fname).encode(), ctypes.byref(h))
        if st != OK:
            raise SurfattError(st, "srcrec_read_csv")
        return cls(h)

    @classmethod
    def from_arrays(cls, evtname, staname, stla, stlo, evla, evlo, period, tt, weight=None):
        n = len(tt)
        enc = lambda names: (ctypes.c_char_p * n)(*[str(v).encode() for v in names])
        keep = [_c64(a) for a in (stla, stlo, evla, evlo, period, tt)]
        w = None if weight is None else _c64(weight)
        h = ctypes.c_void_p()
        L = lib()
        L.surfatt_srcrec_create.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p] + \
            [_dp] * 7 + [ctypes.POINTER(ctypes.c_void_p)]
        st = L.surfatt_srcrec_create(n, enc(evtname), enc(staname), *[_d(a) for a in keep],
                                     _d(w) if w is not None else None, ctypes.byref(h))
        if st != OK:
            raise SurfattError(st, "srcrec_create")
        return cls(h)

    def close(self):
        if self._h:
            L = lib()
            L.surfatt_srcrec_destroy.argtypes = [ctypes.c_void_p]
            L.surfatt_srcrec_destroy.restype = None
            L.surfatt_srcrec_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        a, b, c, d = (ctypes.c_int(0) for _ in range(4))
        L = lib()
        L.surfatt_srcrec_info.argtypes = [ctypes.c_void_p] + [_ip] * 4
        L.surfatt_srcrec_info(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                              ctypes.byref(d))
        return dict(npath=a.value, nperiod=b.value, nsta=c.value, nsolve=d.value)

    def periods(self):
        out = np.zeros(self.info()["nperiod"])
        L = lib()
        L.surfatt_srcrec_periods.argtypes = [ctypes.c_void_p, _dp]
        L.surfatt_srcrec_periods(self._h, _d(out))
        return out

    def stations(self):
        """(names, lon, lat) of the station table."""
        n = self.info()["nsta"]
        lo, la = np.zeros(n), np.zeros(n)
        L = lib()
        L.surfatt_srcrec_stations.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.surfatt_srcrec_stations(self._h, _d(lo), _d(la))
        L.surfatt_srcrec_station_name.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.surfatt_srcrec_station_name.restype = ctypes.c_char_p
        names = [L.surfatt_srcrec_station_name(self._h, i).decode() for i in range(n)]
        return names, lo, la

    def paths(self):
        n = self.info()["npath"]
        d = {k: np.zeros(n) for k in ("tt", "weight", "period")}
        i = {k: np.zeros(n, np.int32) for k in ("evt_station", "station", "period_index")}
        L = lib()
        L.surfatt_srcrec_paths.argtypes = [ctypes.c_void_p] + [_dp] * 3 + [_ip] * 3
        L.surfatt_srcrec_paths(self._h, _d(d["tt"]), _d(d["weight"]), _d(d["period"]),
                               i["evt_station"].ctypes.data_as(_ip),
                               i["station"].ctypes.data_as(_ip),
                               i["period_index"].ctypes.data_as(_ip))
        d.update(i)
        return d

    def build_worklist(self, device=0):
        ns = ctypes.c_int(0)
        L = lib()
        L.surfatt_srcrec_build_worklist.argtypes = [ctypes.c_void_p, ctypes.c_int, _ip]
        st = L.surfatt_srcrec_build_worklist(self._h, int(device), ctypes.byref(ns))
        if st != OK:
            raise SurfattError(st, "srcrec_build_worklist")
        return ns.value

    def worklist(self):
        """The built work list: pidx, sta, srcx, srcy, rec_off, nrec (per
        solve) and recx, recy, tt, weight, path (per receiver)."""
        info = self.info()
        ns, n = info["nsolve"], info["npath"]
        if ns < 0:
            raise SurfattError(BAD_ARG, "srcrec_worklist: build_worklist first")
        wi = {k: np.zeros(ns, np.int32) for k in ("pidx", "sta", "rec_off", "nrec")}
        wd = {k: np.zeros(ns) for k in ("srcx", "srcy")}
        nr = 0
        L = lib()
        L.surfatt_srcrec_worklist.argtypes = [ctypes.c_void_p] + [_ip, _ip, _dp, _dp, _ip, _ip,
                                                                  _dp, _dp, _dp, _dp, _ip]
        L.surfatt_srcrec_worklist(self._h, _i(wi["pidx"]), _i(wi["sta"]), _d(wd["srcx"]),
                                  _d(wd["srcy"]), _i(wi["rec_off"]), _i(wi["nrec"]), None, None,
                                  None, None, None)
        nr = int(wi["nrec"].sum())
        rd = {k: np.zeros(nr) for k in ("recx", "recy", "tt", "weight")}
        rp = np.zeros(nr, np.int32)
        L.surfatt_srcrec_worklist(self._h, None, None, None, None, None, None, _d(rd["recx"]),
                                  _d(rd["recy"]), _d(rd["tt"]), _d(rd["weight"]), _i(rp))
        out = dict(wi, **wd, **rd)
        out["path"] = rp
        return out

    def build_timing(self):
        ms, n = ctypes.c_double(0), ctypes.c_int(0)
        L = lib()
        L.surfatt_srcrec_build_timing.argtypes = [ctypes.c_void_p, _dp, _ip]
        st = L.surfatt_srcrec_build_timing(self._h, ctypes.byref(ms), ctypes.byref(n))
        if st != OK:
            raise SurfattError(st, "srcrec_build_timing")
        return ms.value, n.value

    def write_csv(self, fname, tt_fwd):
        tt_fwd = _c64(tt_fwd)
        L = lib()
        L.surfatt_srcrec_write_csv.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _dp]
        st = L.surfatt_srcrec_write_csv(self._h, str(fname).encode(), _d(tt_fwd))
        if st != OK:
            raise SurfattError(st, "srcrec_write_csv")

    def problem(self, grids, fields, mode=MODE_2D, name="src_rec"):
        """A workloads.Problem whose work list is this table's (built on
        the GPU): grids[p] = (xx, yy) and fields[p] = dict(svel, m11, m12,
        m22) of period p (the table's periods, ascending)."""
        from . import workloads as W
        wl = self.worklist()
        nsolve = len(wl["pidx"])
        solves = []
        for s in range(nsolve):
            r0, nr = int(wl["rec_off"][s]), int(wl["nrec"][s])
            solves.append((int(wl["pidx"][s]), float(wl["srcx"][s]), float(wl["srcy"][s]),
                           wl["recx"][r0:r0 + nr], wl["recy"][r0:r0 + nr],
                           wl["tt"][r0:r0 + nr], wl["weight"][r0:r0 + nr]))
        pb = W._pack(name, grids, fields, solves, self.periods(), mode)
        pb.path = wl["path"].astype(np.int32)
        pb.n_paths = self.info()["npath"]
        return pb


def _i(a):
    return a.ctypes.data_as(_ip)


# ---------------------------------------------------------------------------
# att_measadj mirror (src/measadj.f90)
# ---------------------------------------------------------------------------
class MeasAdj:
    """One (period, source) measurement: get_recs / run_forward / run_adjoint /
    run_adjoint_density / to_table, as in src/measadj.f90:25-114."""

    def __init__(self, xgrids, ygrids, srcx, srcy, recx, recy, tt, weight, idx_path=None):
        self.xgrids, self.ygrids = _c64(xgrids), _c64(ygrids)
        self.srcx, self.srcy = float(srcx), float(srcy)
        self.recx, self.recy, self.tt = _c64(recx), _c64(recy), _c64(tt)
        self.weight = _c64(weight).copy()
        self.nrec = len(self.tt)
        self.idx_path = np.arange(self.nrec) if idx_path is None else np.asarray(idx_path)
        self.timetable = None
        self.tekio = None
        self.chi = None

    def run_forward(self, vel2d, m11, m22, m12):
        nx, ny = len(self.xgrids), len(self.ygrids)
        self.timetable = np.zeros((nx, ny), order="F")
        self.tekio = np.zeros(self.nrec)
        chi = ctypes.c_double(0)
        vel2d, m11, m22, m12 = (_f2(v) for v in (vel2d, m11, m22, m12))
        st = lib().surfatt_measadj_run_forward(
            _d(self.xgrids), _d(self.ygrids), nx, ny, _d(vel2d), _d(m11), _d(m22), _d(m12),
            self.srcx, self.srcy, self.nrec, _d(self.recx), _d(self.recy), _d(self.tt),
            _d(self.weight), _d(self.timetable), _d(self.tekio), ctypes.byref(chi))
        if st not in (OK, NOT_CONVERGED):
            raise SurfattError(st, "run_forward")
        self.chi = chi.value
        return st

    def run_adjoint(self, m11, m22, m12):
        nx, ny = len(self.xgrids), len(self.ygrids)
        adj = np.zeros((nx, ny), order="F")
        m11, m22, m12 = (_f2(v) for v in (m11, m22, m12))
        st = lib().surfatt_measadj_run_adjoint(
            _d(self.xgrids), _d(self.ygrids), nx, ny, _d(m11), _d(m22), _d(m12), self.srcx,
            self.srcy, self.nrec, _d(self.recx), _d(self.recy), _d(self.tt), _d(self.tekio),
            _d(self.weight), _d(_f2(self.timetable)), _d(adj))
        if st not in (OK, NOT_CONVERGED):
            raise SurfattError(st, "run_adjoint")
        return adj

    def run_adjoint_density(self, m11, m22, m12):
        nx, ny = len(self.xgrids), len(self.ygrids)
        den = np.zeros((nx, ny), order="F")
        m11, m22, m12 = (_f2(v) for v in (m11, m22, m12))
        st = lib().surfatt_measadj_run_adjoint_density(
            _d(self.xgrids), _d(self.ygrids), nx, ny, _d(m11), _d(m22), _d(m12), self.srcx,
            self.srcy, self.nrec, _d(self.recx), _d(self.recy), _d(self.weight),
            _d(_f2(self.timetable)), _d(den))
        if st not in (OK, NOT_CONVERGED):
            raise SurfattError(st, "run_adjoint_density")
        return den

    def to_table(self, tt_fwd):
        tt_fwd[self.idx_path] = self.tekio


# ---------------------------------------------------------------------------
# batched engine
# ---------------------------------------------------------------------------
class _CProblem(ctypes.Structure):
    _fields_ = [("nperiod", ctypes.c_int), ("nx", _ip), ("ny", _ip), ("xoff", _llp),
                ("yoff", _llp), ("goff", _llp), ("xgrid", _dp), ("ygrid", _dp),
                ("svel", _dp), ("m11", _dp), ("m12", _dp), ("m22", _dp),
                ("nsolve", ctypes.c_int), ("pidx", _ip), ("srcx", _dp), ("srcy", _dp),
                ("rec_off", _ip), ("nrec", _ip), ("recx", _dp), ("recy", _dp), ("tt", _dp),
                ("weight", _dp), ("path", _ip), ("npath", ctypes.c_int)]


class _CResult(ctypes.Structure):
    _fields_ = [("adj_s", _dp), ("adj_density", _dp), ("chi", _dp), ("tt_fwd", _dp),
                ("status", _ip), ("fwd_iters", _ip), ("adj_iters", _ip)]


def pack_problem(pb, keep):
    """ctypes view of a workloads.Problem (arrays kept alive in `keep`)."""

    def P(a, kind):
        a = np.ascontiguousarray(a, dtype={"d": np.float64, "i": np.int32, "q": np.int64}[kind])
        keep.append(a)
        return a.ctypes.data_as({"d": _dp, "i": _ip, "q": _llp}[kind])

    return _CProblem(pb.nperiod, P(pb.nx, "i"), P(pb.ny, "i"), P(pb.xoff, "q"), P(pb.yoff, "q"),
                     P(pb.goff, "q"), P(pb.xgrid, "d"), P(pb.ygrid, "d"), P(pb.svel, "d"),
                     P(pb.m11, "d"), P(pb.m12, "d"), P(pb.m22, "d"), pb.nsolve, P(pb.pidx, "i"),
                     P(pb.srcx, "d"), P(pb.srcy, "d"), P(pb.rec_off, "i"), P(pb.nrec, "i"),
                     P(pb.recx, "d"), P(pb.recy, "d"), P(pb.tt, "d"), P(pb.weight, "d"),
                     P(pb.path, "i"), pb.npath)


class _DeviceArray:
    """A float64 vector in device memory, exposed to torch through the CUDA
    array interface (zero copy)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": "<f8",
                                         "data": (int(ptr), False), "version": 2,
                                         "strides": None}


class Engine:
    """Batched gradient evaluations on one GPU (device-resident problem)."""

    def __init__(self, device=0, hbm_budget_bytes=0):
        self._h = ctypes.c_void_p()
        st = lib().surfatt_engine_create(ctypes.byref(self._h), device, hbm_budget_bytes)
        if st != OK:
            raise SurfattError(st, "engine_create")
        self.pb = None

    def close(self):
        if self._h:
            lib().surfatt_engine_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, pb):
        keep = []
        cp = pack_problem(pb, keep)
        st = lib().surfatt_engine_load(self._h, ctypes.byref(cp))
        if st != OK:
            raise SurfattError(st, "engine_load")
        self.pb = pb

    def update_velocity(self, svel):
        svel = _c64(svel)
        st = lib().surfatt_engine_update_velocity(self._h, _d(svel))
        if st != OK:
            raise SurfattError(st, "engine_update_velocity")

    def run(self, mode=MODE_2D, precision=PREC_FP64):
        st = lib().surfatt_engine_run(self._h, int(mode), int(precision))
        if st != OK:
            raise SurfattError(st, "engine_run")

    def sync(self):
        return lib().surfatt_engine_sync(self._h)

    def results(self, adj=True, density=True, tt=True, per_solve=True, into=None):
        """Copy the last run's results to host arrays (new arrays, or the
        preallocated ones of `into`, e.g. pinned buffers)."""
        pb = self.pb
        out = {}
        r = _CResult()
        keep = []

        def buf(name, n, dt):
            if into is not None and name in into:
                a = into[name]
                assert a.dtype == dt and a.flags.c_contiguous and a.size >= max(n, 1)
            else:
                a = np.zeros(max(n, 1), dt)
            keep.append(a)
            out[name] = a
            return a.ctypes.data_as(_dp if dt == np.float64 else _ip)

        chi = into["chi"] if into is not None and "chi" in into else np.zeros(1)
        out["chi"] = chi
        r.chi = chi.ctypes.data_as(_dp)
        if adj:
            r.adj_s = buf("adj_s", pb.ncell, np.float64)
        if density:
            r.adj_density = buf("adj_density", pb.ncell, np.float64)
        if tt:
            r.tt_fwd = buf("tt_fwd", pb.npath, np.float64)
        if per_solve:
            r.status = buf("status", pb.nsolve, np.int32)
            r.fwd_iters = buf("fwd_iters", pb.nsolve, np.int32)
            r.adj_iters = buf("adj_iters", pb.nsolve, np.int32)
        st = lib().surfatt_engine_results(self._h, ctypes.byref(r))
        if st != OK:
            raise SurfattError(st, "engine_results")
        out["chi"] = float(chi[0])
        if tt:
            out["tt_fwd"] = out["tt_fwd"][:pb.npath]
        return out

    def timing(self):
        t, k, n = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_int(0)
        st = lib().surfatt_engine_timing(self._h, ctypes.byref(t), ctypes.byref(k),
                                         ctypes.byref(n))
        if st != OK:
            raise SurfattError(st, "engine_timing")
        return t.value, k.value, n.value

    def launch_config(self):
        g, b, n = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        sm = ctypes.c_size_t(0)
        L = lib()
        L.surfatt_engine_launch_config.argtypes = [ctypes.c_void_p, _ip, _ip, _ip,
                                                   ctypes.POINTER(ctypes.c_size_t)]
        st = L.surfatt_engine_launch_config(self._h, ctypes.byref(g), ctypes.byref(b),
                                            ctypes.byref(n), ctypes.byref(sm))
        if st != OK:
            raise SurfattError(st, "engine_launch_config")
        return dict(grid=g.value, block=b.value, blocks_per_sm=n.value, smem_bytes=sm.value)

    def autotune(self, mode=MODE_2D, precision=PREC_FP32):
        """Time the applicable kernel variants and keep the fastest."""
        L = lib()
        L.surfatt_engine_autotune.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _ip,
                                              _ip, _dp]
        k, v, ms = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0)
        st = L.surfatt_engine_autotune(self._h, int(mode), int(precision), ctypes.byref(k),
                                       ctypes.byref(v), ctypes.byref(ms))
        if st != OK:
            raise SurfattError(st, "engine_autotune")
        return dict(kind=k.value, variant=v.value, kernel_ms=ms.value)

    def kernel_variant(self):
        L = lib()
        L.surfatt_engine_kernel_variant.argtypes = [ctypes.c_void_p, _ip, _ip]
        k, v = ctypes.c_int(0), ctypes.c_int(0)
        st = L.surfatt_engine_kernel_variant(self._h, ctypes.byref(k), ctypes.byref(v))
        if st != OK:
            raise SurfattError(st, "engine_kernel_variant")
        return dict(kind=k.value, variant=v.value)

    def set_kernel(self, precision, kind=-1, variant=-1):
        """Fix the solve kernel of later runs (-1: automatic)."""
        L = lib()
        L.surfatt_engine_set_kernel.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 3
        st = L.surfatt_engine_set_kernel(self._h, int(precision), int(kind), int(variant))
        if st != OK:
            raise SurfattError(st, "engine_set_kernel")

    PHASES = ("setup", "forward", "receivers", "adjoint_setup", "adjoint", "slot")

    def set_profile(self, enable):
        """Per-phase cycle counters of the FP32 warp kernel (default off)."""
        L = lib()
        L.surfatt_engine_set_profile.argtypes = [ctypes.c_void_p, ctypes.c_int]
        st = L.surfatt_engine_set_profile(self._h, 1 if enable else 0)
        if st != OK:
            raise SurfattError(st, "engine_set_profile")

    def phase_cycles(self):
        c = np.zeros(len(self.PHASES))
        L = lib()
        L.surfatt_engine_phase_cycles.argtypes = [ctypes.c_void_p, _dp]
        st = L.surfatt_engine_phase_cycles(self._h, _d(c))
        if st != OK:
            raise SurfattError(st, "engine_phase_cycles")
        return dict(zip(self.PHASES, c.tolist()))

    def set_graphs(self, enable):
        """Capture/replay evaluations as CUDA graphs (default on)."""
        L = lib()
        L.surfatt_engine_set_graphs.argtypes = [ctypes.c_void_p, ctypes.c_int]
        st = L.surfatt_engine_set_graphs(self._h, 1 if enable else 0)
        if st != OK:
            raise SurfattError(st, "engine_set_graphs")

    def smooth(self, sigma, host=True):
        """ker_s of tomo2d's optimize step (src/tomo2d.f90:216-222): every
        period's adj_s of the last mode-2/3 run smoothed by
        gaussian_smooth_geo_2 with `sigma` (degrees), on the device.  Returns
        ker_s (ncell, the adj_s layout), or None with host=False (the result
        stays on the device; sync() waits for it)."""
        L = lib()
        L.surfatt_engine_smooth.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp]
        out = np.zeros(self.pb.ncell) if host else None
        st = L.surfatt_engine_smooth(self._h, float(sigma), _d(out) if host else None)
        if st != OK:
            raise SurfattError(st, "engine_smooth")
        return out

    def smooth_timing(self):
        """(kernel ms, window taps, launches) of the last smooth()."""
        L = lib()
        L.surfatt_engine_smooth_timing.argtypes = [ctypes.c_void_p, _dp, _dp, _ip]
        ms, taps, n = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_int(0)
        st = L.surfatt_engine_smooth_timing(self._h, ctypes.byref(ms), ctypes.byref(taps),
                                            ctypes.byref(n))
        if st != OK:
            raise SurfattError(st, "engine_smooth_timing")
        return ms.value, taps.value, n.value

    def set_keep_fields(self, enable):
        """Keep every solve's travel-time field in later runs (default off)."""
        L = lib()
        L.surfatt_engine_set_keep_fields.argtypes = [ctypes.c_void_p, ctypes.c_int]
        st = L.surfatt_engine_set_keep_fields(self._h, 1 if enable else 0)
        if st != OK:
            raise SurfattError(st, "engine_set_keep_fields")

    def fields(self):
        """The last run's travel-time fields, one (nx, ny) array per solve."""
        pb = self.pb
        cells = (pb.nx[pb.pidx].astype(np.int64) * pb.ny[pb.pidx])
        flat = np.zeros(max(int(cells.sum()), 1))
        L = lib()
        L.surfatt_engine_fields.argtypes = [ctypes.c_void_p, _dp]
        st = L.surfatt_engine_fields(self._h, _d(flat))
        if st != OK:
            raise SurfattError(st, "engine_fields")
        out, o = [], 0
        for s in range(pb.nsolve):
            p = int(pb.pidx[s])
            n = int(cells[s])
            out.append(flat[o:o + n].reshape((int(pb.nx[p]), int(pb.ny[p])), order="F"))
            o += n
        return out

    def test_hold(self, solve=-1, wait_polls=0):
        """Test hook of the bounded item wait (solve -1: off)."""
        L = lib()
        L.surfatt_engine_test_hold.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        st = L.surfatt_engine_test_hold(self._h, int(solve), int(wait_polls))
        if st != OK:
            raise SurfattError(st, "engine_test_hold")

    def device_results(self):
        """The last run's adj_s, adj_density, tt_fwd and chi as torch tensors
        that view the engine's device memory (no copy; valid until the next
        load; None where the mode produces no such field).  Call after
        sync().  For the multi-rank sum of the results on the device."""
        import torch
        L = lib()
        L.surfatt_engine_device_results.argtypes = [ctypes.c_void_p] + [
            ctypes.POINTER(ctypes.c_void_p)] * 5
        ptr = [ctypes.c_void_p() for _ in range(5)]
        st = L.surfatt_engine_device_results(self._h, *[ctypes.byref(p) for p in ptr])
        if st != OK:
            raise SurfattError(st, "engine_device_results")
        pb = self.pb
        out = {}
        for name, p, n in (("adj_s", ptr[0], pb.ncell), ("adj_density", ptr[1], pb.ncell),
                           ("tt_fwd", ptr[2], pb.npath), ("chi", ptr[3], 1)):
            out[name] = None if not p.value else torch.as_tensor(_DeviceArray(p.value, n))
        return out

    def work(self):
        f, a = ctypes.c_double(0), ctypes.c_double(0)
        st = lib().surfatt_engine_work(self._h, ctypes.byref(f), ctypes.byref(a))
        if st != OK:
            raise SurfattError(st, "engine_work")
        return f.value, a.value

    def evaluate(self, pb=None, mode=None, precision=PREC_FP64):
        """load (if given) + run + results: one gradient evaluation."""
        if pb is not None:
            self.load(pb)
        mode = self.pb.mode if mode is None else mode
        self.run(mode, precision)
        self.sync()
        return self.results()


# ---------------------------------------------------------------------------
# serving loop
# ---------------------------------------------------------------------------
class _CServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_longlong), ("completed", ctypes.c_longlong),
                ("failed", ctypes.c_longlong), ("solves", ctypes.c_longlong),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double),
                ("mean_ms", ctypes.c_double), ("span_s", ctypes.c_double),
                ("solves_per_s", ctypes.c_double), ("hbm_budget_bytes", ctypes.c_size_t),
                ("hbm_peak_bytes", ctypes.c_size_t), ("inflight_peak", ctypes.c_int)]


class Server:
    """Request loop on one GPU: resident models and work lists, requests
    admitted by an HBM budget and run concurrently (continuous batching)."""

    def __init__(self, device=0, hbm_budget_bytes=8 << 30, max_inflight=4):
        L = lib()
        L.surfatt_server_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                            ctypes.c_size_t, ctypes.c_int]
        L.surfatt_server_destroy.argtypes = [ctypes.c_void_p]
        L.surfatt_server_destroy.restype = None
        L.surfatt_server_add_model.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _ip]
        L.surfatt_server_add_worklist.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                  _ip]
        L.surfatt_server_submit.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, ctypes.c_int,
                                            ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]
        L.surfatt_server_wait.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_double,
                                          ctypes.c_void_p, _dp]
        L.surfatt_server_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.surfatt_server_reset_stats.argtypes = [ctypes.c_void_p]
        self._h = ctypes.c_void_p()
        st = L.surfatt_server_create(ctypes.byref(self._h), device, int(hbm_budget_bytes),
                                     int(max_inflight))
        if st != OK:
            raise SurfattError(st, "server_create")
        self._shape = {}

    def close(self):
        if self._h:
            lib().surfatt_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_model(self, pb):
        keep = []
        cp = pack_problem(pb, keep)
        mid = ctypes.c_int(0)
        st = lib().surfatt_server_add_model(self._h, ctypes.byref(cp), ctypes.byref(mid))
        if st != OK:
            raise SurfattError(st, "server_add_model")
        return mid.value

    def add_worklist(self, model_id, pb):
        keep = []
        cp = pack_problem(pb, keep)
        wid = ctypes.c_int(0)
        st = lib().surfatt_server_add_worklist(self._h, int(model_id), ctypes.byref(cp),
                                               ctypes.byref(wid))
        if st != OK:
            raise SurfattError(st, "server_add_worklist")
        self._shape[wid.value] = (pb.ncell, pb.npath, pb.nsolve)
        return wid.value

    def submit(self, worklist_id, svel=None, mode=MODE_2D, precision=PREC_FP64):
        t = ctypes.c_longlong(0)
        v = None if svel is None else np.ascontiguousarray(svel, dtype=np.float64)
        st = lib().surfatt_server_submit(self._h, int(worklist_id),
                                         None if v is None else _d(v), int(mode), int(precision),
                                         ctypes.byref(t))
        if st != OK:
            raise SurfattError(st, "server_submit")
        return (t.value, worklist_id)

    def wait(self, ticket, timeout_s=0.0):
        """Returns (status, result dict, latency_ms)."""
        tk, wid = ticket
        ncell, npath, nsolve = self._shape[wid]
        out = dict(adj_s=np.zeros(max(ncell, 1)), adj_density=np.zeros(max(ncell, 1)),
                   tt_fwd=np.zeros(max(npath, 1)), chi=np.zeros(1),
                   status=np.zeros(max(nsolve, 1), np.int32),
                   fwd_iters=np.zeros(max(nsolve, 1), np.int32),
                   adj_iters=np.zeros(max(nsolve, 1), np.int32))
        r = _CResult(_d(out["adj_s"]), _d(out["adj_density"]), _d(out["chi"]),
                     _d(out["tt_fwd"]), out["status"].ctypes.data_as(_ip),
                     out["fwd_iters"].ctypes.data_as(_ip), out["adj_iters"].ctypes.data_as(_ip))
        lat = ctypes.c_double(0)
        st = lib().surfatt_server_wait(self._h, tk, float(timeout_s), ctypes.byref(r),
                                       ctypes.byref(lat))
        out["chi"] = float(out["chi"][0])
        out["tt_fwd"] = out["tt_fwd"][:npath]
        return st, out, lat.value

    def stats(self):
        s = _CServerStats()
        st = lib().surfatt_server_stats(self._h, ctypes.byref(s))
        if st != OK:
            raise SurfattError(st, "server_stats")
        return {f: getattr(s, f) for f, _ in _CServerStats._fields_}

    def reset_stats(self):
        lib().surfatt_server_reset_stats(self._h)
