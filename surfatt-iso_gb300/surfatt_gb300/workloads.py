"""Synthetic SurfATT workloads: packed (period, source) work lists.

A ``Problem`` is one gradient evaluation of the travel-time + adjoint path, in
the layout the batched library consumes:

* periods: period ``p`` has its own lon/lat grid of ``nx[p] x ny[p]`` nodes
  (coordinates ``xgrid[xoff[p]:]``, ``ygrid[yoff[p]:]`` in degrees) and
  fields ``svel`` (phase velocity, km/s), ``m11``, ``m12``, ``m22`` (surface
  metric) stored column-major (x fastest) at cell offset ``goff[p]``.  This
  is the reference's ``att_grid`` (src/grid.f90:25-33) with the period index
  moved from fastest to slowest so that every solve reads contiguous planes.
* solves: solve ``s`` is (period ``pidx[s]``, source ``srcx/srcy[s]``) with
  receivers ``rec_off[s] .. rec_off[s]+nrec[s]-1`` of the receiver table
  (``recx, recy, tt, weight, path``); this is ``SrcRec%isrcs`` plus the
  per-source gathers of ``get_evt_gather`` (src/src_rec.f90:252-283, 338-369).

The generators follow the reference's formulas where it has them
(checkerboard: src/acqui_2d.f90:101-147, grid: src/model.f90:52-77).  The
public benchmark datasets of the reference's papers are not available; every
workload here is seeded synthetic data with the shapes and value ranges of
the configurations it is named after.
"""
from __future__ import annotations

import csv
import dataclasses
import math

import numpy as np

# shared_par.f90:11 pi = 3.14159265359 is a default-real literal (single-rounded)
PI_F = float(np.float32(3.14159265359))
R_EARTH = 6371.0


@dataclasses.dataclass
class Problem:
    name: str
    nperiod: int
    nx: np.ndarray
    ny: np.ndarray
    xoff: np.ndarray
    yoff: np.ndarray
    goff: np.ndarray
    xgrid: np.ndarray
    ygrid: np.ndarray
    svel: np.ndarray
    m11: np.ndarray
    m12: np.ndarray
    m22: np.ndarray
    pidx: np.ndarray
    srcx: np.ndarray
    srcy: np.ndarray
    rec_off: np.ndarray
    nrec: np.ndarray
    recx: np.ndarray
    recy: np.ndarray
    tt: np.ndarray
    weight: np.ndarray
    path: np.ndarray
    periods: np.ndarray
    mode: int = 2  # 2: tomo2d (adj/svel^2), 3: 3-D (adj, density /svel^3)
    n_paths: int = -1  # size of the synthetic-time table (default: len(path))

    @property
    def nsolve(self) -> int:
        return int(len(self.pidx))

    @property
    def npath(self) -> int:
        return int(self.n_paths) if self.n_paths >= 0 else int(len(self.path))

    @property
    def ncell(self) -> int:
        return int(self.goff[-1] + self.nx[-1] * self.ny[-1]) if self.nperiod else 0

    def field(self, name: str, p: int) -> np.ndarray:
        """(nx, ny) view of a per-period field (Fortran order)."""
        a = getattr(self, name)
        nx, ny, g = int(self.nx[p]), int(self.ny[p]), int(self.goff[p])
        return a[g:g + nx * ny].reshape((nx, ny), order="F")

    def grid(self, p: int):
        nx, ny = int(self.nx[p]), int(self.ny[p])
        return (self.xgrid[self.xoff[p]:self.xoff[p] + nx],
                self.ygrid[self.yoff[p]:self.yoff[p] + ny])

    def cell_updates_per_iteration(self) -> np.ndarray:
        """nx*ny per solve (one forward sweep pass = 4 * nx * ny cell visits)."""
        return (self.nx[self.pidx].astype(np.int64) * self.ny[self.pidx])

    def subset(self, solves) -> "Problem":
        """A problem with the same periods and only the listed solves (in order)."""
        solves = np.asarray(solves, dtype=np.int64)
        offs, recs = [], []
        o = 0
        for s in solves:
            r0, n = int(self.rec_off[s]), int(self.nrec[s])
            recs.append(np.arange(r0, r0 + n))
            offs.append(o)
            o += n
        ridx = np.concatenate(recs) if recs else np.zeros(0, np.int64)
        return dataclasses.replace(
            self, pidx=self.pidx[solves].copy(), srcx=self.srcx[solves].copy(),
            srcy=self.srcy[solves].copy(), rec_off=np.asarray(offs, np.int32),
            nrec=self.nrec[solves].copy(), recx=self.recx[ridx].copy(),
            recy=self.recy[ridx].copy(), tt=self.tt[ridx].copy(),
            weight=self.weight[ridx].copy(), path=np.arange(len(ridx), dtype=np.int32),
            n_paths=-1)


def _pack(name, grids, fields, solves, periods, mode):
    """grids: list of (xx, yy); fields: list of dict(svel, m11, m12, m22) (nx, ny);
    solves: list of (p, sx, sy, recx[], recy[], tt[], weight[])."""
    nx = np.array([len(g[0]) for g in grids], np.int32)
    ny = np.array([len(g[1]) for g in grids], np.int32)
    xoff = np.concatenate([[0], np.cumsum(nx)[:-1]]).astype(np.int64)
    yoff = np.concatenate([[0], np.cumsum(ny)[:-1]]).astype(np.int64)
    goff = np.concatenate([[0], np.cumsum(nx.astype(np.int64) * ny)[:-1]]).astype(np.int64)
    cat = lambda k: np.concatenate([np.asarray(f[k], np.float64).ravel(order="F") for f in fields])
    nrec = np.array([len(s[3]) for s in solves], np.int32)
    rec_off = np.concatenate([[0], np.cumsum(nrec)[:-1]]).astype(np.int32)
    return Problem(
        name=name, nperiod=len(grids), nx=nx, ny=ny, xoff=xoff, yoff=yoff, goff=goff,
        xgrid=np.concatenate([g[0] for g in grids]).astype(np.float64),
        ygrid=np.concatenate([g[1] for g in grids]).astype(np.float64),
        svel=cat("svel"), m11=cat("m11"), m12=cat("m12"), m22=cat("m22"),
        pidx=np.array([s[0] for s in solves], np.int32),
        srcx=np.array([s[1] for s in solves], np.float64),
        srcy=np.array([s[2] for s in solves], np.float64),
        rec_off=rec_off, nrec=nrec,
        recx=np.concatenate([s[3] for s in solves]).astype(np.float64),
        recy=np.concatenate([s[4] for s in solves]).astype(np.float64),
        tt=np.concatenate([s[5] for s in solves]).astype(np.float64),
        weight=np.concatenate([s[6] for s in solves]).astype(np.float64),
        path=np.arange(int(nrec.sum()), dtype=np.int32),
        periods=np.asarray(periods, np.float64), mode=mode)


def arange_grid(beg: float, n: int, d: float) -> np.ndarray:
    """xgrids = arange(xbeg, xend, d) = xbeg + i*d (src/shared/utils.f90:645-653)."""
    return beg + np.arange(n, dtype=np.float64) * d


def checkerboard_2d(nx: int, ny: int, npx: int, npy: int, amp: float, hmarg_cells: int = 0):
    """Multiplier (1 + amp * sin(npx*pi*i/n) * sin(npy*pi*j/n)), i, j = 1..n
    (att_acqui_2d_add_pert, src/acqui_2d.f90:124-140, with hmarg = 0)."""
    i = np.arange(1, nx - 2 * hmarg_cells + 1, dtype=np.float64)
    j = np.arange(1, ny - 2 * hmarg_cells + 1, dtype=np.float64)
    xp = np.zeros(nx)
    yp = np.zeros(ny)
    xp[hmarg_cells:nx - hmarg_cells] = np.sin(npx * PI_F * i / (nx - 2 * hmarg_cells))
    yp[hmarg_cells:ny - hmarg_cells] = np.sin(npy * PI_F * j / (ny - 2 * hmarg_cells))
    return 1.0 + amp * xp[:, None] * yp[None, :]


def gps2dist(lat1, lon1, lat2, lon2):
    """Great-circle distance in km (haversine)."""
    p1, p2 = np.radians(lat1), np.radians(lat2)
    dl = np.radians(np.asarray(lon2) - np.asarray(lon1))
    a = np.sin((p2 - p1) / 2) ** 2 + np.cos(p1) * np.cos(p2) * np.sin(dl / 2) ** 2
    return 2 * R_EARTH * np.arcsin(np.sqrt(np.minimum(a, 1.0)))


def _stations(rng, n, x0, x1, y0, y1, frac=0.8):
    """n stations uniform in the interior `frac` box of [x0,x1]x[y0,y1]."""
    mx = (x1 - x0) * (1 - frac) / 2
    my = (y1 - y0) * (1 - frac) / 2
    return rng.uniform(x0 + mx, x1 - mx, n), rng.uniform(y0 + my, y1 - my, n)


def _flat_metric(nx, ny):
    return np.ones((nx, ny)), np.zeros((nx, ny)), np.ones((nx, ny))


def _all_pairs(p, sx, sy, tt_fn, weight=1.0):
    """Each station a source, the other stations its receivers."""
    out = []
    n = len(sx)
    for s in range(n):
        r = np.array([k for k in range(n) if k != s])
        out.append((p, sx[s], sy[s], sx[r], sy[r], tt_fn(s, r), np.full(len(r), weight)))
    return out


def flat_case(nx=33, ny=29, d=0.05, nsta=6, nperiod=1, seed=7, vel=3.0, pert=0.06,
              mode=2, x0=100.0, y0=22.0, name="flat_case"):
    """Small lon/lat case on one grid: checkerboard velocity, flat metric,
    `nsta` stations each a source for every period; observed times are the
    great-circle distance over `vel` times (1 + 2% seeded noise)."""
    rng = np.random.default_rng(seed)
    xx, yy = arange_grid(x0, nx, d), arange_grid(y0, ny, d)
    sx, sy = _stations(rng, nsta, xx[0], xx[-1], yy[0], yy[-1])
    grids, fields, solves = [], [], []
    for p in range(nperiod):
        m11, m12, m22 = _flat_metric(nx, ny)
        sv = vel * (1 + 0.02 * p) * checkerboard_2d(nx, ny, 2, 3, pert)
        grids.append((xx, yy))
        fields.append(dict(svel=sv, m11=m11, m12=m12, m22=m22))
        noise = rng.normal(0, 0.02, (nsta, nsta))
        tt_fn = lambda s, r: gps2dist(sy[s], sx[s], sy[r], sx[r]) / vel * (1 + noise[s, r])
        solves += _all_pairs(p, sx, sy, tt_fn)
    return _pack(name, grids, fields, solves, np.arange(1, nperiod + 1) * 10.0, mode)


def config1(observed_tt=None):
    """Plain FP64 CPU-runnable case (seed 0): 81x81 nodes at 0.05 deg
    (lon 100-104, lat 22-26); 25 stations uniform in the interior 80 %; each
    station a source, the other 24 its receivers (600 paths); one period
    (10 s); starting model 3.0 km/s; 2-D mode (adj / svel^2).  The observed
    times come from a forward run on the +-6 % 2x3 checkerboard model
    (``observed_tt``, 600 values in solve order, e.g. from the committed
    fixture); without them the straight-ray time on that model is used."""
    rng = np.random.default_rng(0)
    n, d = 81, 0.05
    xx, yy = arange_grid(100.0, n, d), arange_grid(22.0, n, d)
    sx, sy = _stations(rng, 25, xx[0], xx[-1], yy[0], yy[-1])
    m11, m12, m22 = _flat_metric(n, n)
    sv = np.full((n, n), 3.0)
    if observed_tt is None:
        obs = lambda s, r: gps2dist(sy[s], sx[s], sy[r], sx[r]) / 3.0
    else:
        obs_all = np.asarray(observed_tt, np.float64).reshape(25, 24)
        obs = lambda s, r: obs_all[s]
    solves = _all_pairs(0, sx, sy, obs)
    return _pack("config1_81x81_25sta", [(xx, yy)], [dict(svel=sv, m11=m11, m12=m12, m22=m22)],
                 solves, [10.0], 2)


def config1_true_model():
    """The +-6 % 2x3 checkerboard model that generates config 1's observed times."""
    pb = config1()
    pb.svel = (3.0 * checkerboard_2d(81, 81, 2, 3, 0.06)).ravel(order="F")
    return pb


def _vs_column_average(vs_top, vs_bot, ztop, zbot, depth_km):
    """Depth average of a linear Vs(z) over [0, depth]."""
    d = np.minimum(depth_km, zbot)
    return vs_top + (vs_bot - vs_top) * (d / 2) / (zbot - ztop)


def config2(nsta=80, nperiod=16, n=120, d=0.05, seed=1, mode=3, name=None):
    """3-D-iso gradient evaluation (seed 1): Vs 3.2->4.5 km/s linear over
    0-60 km (30 nodes) plus a +-5 % 2x3x2 checkerboard, 16 periods
    log-spaced 2-40 s, 80 random stations as sources (80x79 paths per
    period), forward grid 120x120 at 0.05 deg, 3-D mode (two adjoints per
    solve, adj and density / svel^3).  The dispersion step (surfdisp96) is
    out of scope, so the phase velocity of period T is the proxy
    0.92 * mean(Vs over 0 .. 0.4*lambda), lambda = 3.5 km/s * T, evaluated
    on the 30 depth nodes.  Observed times: great-circle distance over the
    period's mean phase velocity, times (1 + 3 % seeded noise)."""
    rng = np.random.default_rng(seed)
    xx, yy = arange_grid(100.0, n, d), arange_grid(22.0, n, d)
    z = np.linspace(0.0, 60.0, 30)
    vs1d = 3.2 + (4.5 - 3.2) * z / 60.0
    kz = np.arange(1, 31)
    cbz = np.sin(2 * PI_F * kz / 30)
    cbxy = checkerboard_2d(n, n, 2, 3, 1.0) - 1.0   # sin * sin
    periods = np.geomspace(2.0, 40.0, nperiod)
    sx, sy = _stations(rng, nsta, xx[0], xx[-1], yy[0], yy[-1])
    grids, fields, solves = [], [], []
    dist = gps2dist(sy[:, None], sx[:, None], sy[None, :], sx[None, :])
    for p, T in enumerate(periods):
        lam = 3.5 * T
        sel = z <= max(0.4 * lam, z[1])
        wz = sel / sel.sum()
        c1d = 0.92 * float((vs1d * wz).sum())
        pert = 0.05 * float((vs1d * cbz * wz).sum()) / float((vs1d * wz).sum())
        sv = c1d * (1 + pert * cbxy)
        m11, m12, m22 = _flat_metric(n, n)
        grids.append((xx, yy))
        fields.append(dict(svel=sv, m11=m11, m12=m12, m22=m22))
        noise = rng.normal(0, 0.03, (nsta, nsta))
        tt_fn = lambda s, r, c=c1d, nz=noise: dist[s, r] / c * (1 + nz[s, r])
        solves += _all_pairs(p, sx, sy, tt_fn)
    return _pack(name or f"config2_{n}x{n}_{nsta}sta_{nperiod}per", grids, fields, solves,
                 periods, mode)


def gaussian_random_field(rng, nx, ny, dx_km, dy_km, corr_km, sigma):
    """Zero-mean field with Gaussian correlation `corr_km` and std `sigma`,
    by FFT filtering of white noise."""
    w = rng.standard_normal((nx, ny))
    kx = np.fft.fftfreq(nx, d=dx_km) * 2 * np.pi
    ky = np.fft.fftfreq(ny, d=dy_km) * 2 * np.pi
    filt = np.exp(-0.25 * corr_km ** 2 * (kx[:, None] ** 2 + ky[None, :] ** 2))
    f = np.real(np.fft.ifft2(np.fft.fft2(w) * filt))
    f -= f.mean()
    s = f.std()
    return f * (sigma / s) if s > 0 else f


def config4(nsrc=120, nperiod=25, nmax=384, nmin=64, span_deg=8.0, seed=3, mode=3, name=None):
    """Batched uneven grids (seed 3): 120 sources x 25 periods (3000 solves);
    period p (log-spaced 2-50 s) gets an n_p x n_p grid over the same
    8 x 8 deg box, n_p geometric from 384 down to 64 and rounded to a
    multiple of 8 (coarser for longer periods); velocity 3.5 km/s times
    (1 + Gaussian random field, sigma 4 %, correlation 30 km); flat metric.
    Each source has the other 119 stations as receivers."""
    rng = np.random.default_rng(seed)
    periods = np.geomspace(2.0, 50.0, nperiod)
    sides = np.geomspace(nmax, nmin, nperiod)
    sides = (np.round(sides / 8) * 8).astype(int)
    x0, y0 = 96.0, 20.0
    sx, sy = _stations(rng, nsrc, x0, x0 + span_deg, y0, y0 + span_deg)
    dist = gps2dist(sy[:, None], sx[:, None], sy[None, :], sx[None, :])
    grids, fields, solves = [], [], []
    km_per_deg = R_EARTH * math.pi / 180
    for p in range(nperiod):
        n = int(sides[p])
        d = span_deg / (n - 1)
        xx, yy = arange_grid(x0, n, d), arange_grid(y0, n, d)
        grf = gaussian_random_field(rng, n, n, d * km_per_deg * math.cos(math.radians(y0 + 4)),
                                    d * km_per_deg, 30.0, 0.04)
        sv = 3.5 * (1 + grf)
        m11, m12, m22 = _flat_metric(n, n)
        grids.append((xx, yy))
        fields.append(dict(svel=sv, m11=m11, m12=m12, m22=m22))
        noise = rng.normal(0, 0.03, (nsrc, nsrc))
        tt_fn = lambda s, r, nz=noise: dist[s, r] / 3.5 * (1 + nz[s, r])
        solves += _all_pairs(p, sx, sy, tt_fn)
    return _pack(name or f"config4_{nsrc}src_{nperiod}per_{nmin}-{nmax}", grids, fields,
                 solves, periods, mode)


def topo_metric(topo_km, xx, yy):
    """Surface metric of src/grid.f90:117-122 from a topography grid (km):
    fx, fy = topography gradients in km/km (geographic, gradient_2_geo),
    a = (1+fy^2)/(1+fx^2+fy^2), b = (1+fx^2)/(...), c = fx*fy/(...);
    m11 = a, m22 = b, m12 = -c (src/grid.f90:142-145)."""
    km_per_deg = R_EARTH * math.pi / 180
    dxk = (xx[1] - xx[0]) * km_per_deg * np.cos(np.radians(yy))[None, :]
    dyk = (yy[1] - yy[0]) * km_per_deg
    fx = np.gradient(topo_km, axis=0) / dxk
    fy = np.gradient(topo_km, axis=1) / dyk
    den = 1 + fx ** 2 + fy ** 2
    a = (1 + fy ** 2) / den
    b = (1 + fx ** 2) / den
    c = fx * fy / den
    return a, -c, b


def config5_model(n_lon=150, n_lat=200, d=0.02, seed=4):
    """Curved-surface model (seed 4): Gaussian island bump (peak 4 km, radius
    40 km) plus 200 m random-field roughness on a 150x200 grid at 0.02 deg.
    Returns (xx, yy, topo_km, m11, m12, m22)."""
    rng = np.random.default_rng(seed)
    xx, yy = arange_grid(-156.5, n_lon, d), arange_grid(18.0, n_lat, d)
    km_per_deg = R_EARTH * math.pi / 180
    X = (xx[:, None] - xx.mean()) * km_per_deg * math.cos(math.radians(yy.mean()))
    Y = (yy[None, :] - yy.mean()) * km_per_deg
    topo = 4.0 * np.exp(-(X ** 2 + Y ** 2) / (2 * 40.0 ** 2))
    topo = topo + gaussian_random_field(rng, n_lon, n_lat, d * km_per_deg, d * km_per_deg,
                                        5.0, 0.2)
    m11, m12, m22 = topo_metric(topo, xx, yy)
    return xx, yy, topo, m11, m12, m22


# ----------------------------------------------------------------------------
# src_rec CSV (src/src_rec.f90:285-325 column set)
# ----------------------------------------------------------------------------
SRC_REC_HEADER = ["tt", "staname", "stla", "stlo", "stel", "evtname", "evla", "evlo", "evel",
                  "period", "weight", "dist", "vel"]


def write_src_rec_csv(fname, pb: Problem, tt=None, names=None):
    """Write a problem's paths in the reference's src_rec CSV layout."""
    tt = pb.tt if tt is None else tt
    with open(fname, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(SRC_REC_HEADER)
        for s in range(pb.nsolve):
            r0, nr = int(pb.rec_off[s]), int(pb.nrec[s])
            ev = names[s] if names else f"EV{s:04d}"
            for i in range(nr):
                k = r0 + i
                dist = float(gps2dist(pb.srcy[s], pb.srcx[s], pb.recy[k], pb.recx[k]))
                w.writerow([f"{tt[pb.path[k]]:.6f}", f"ST{k:05d}", f"{pb.recy[k]:.4f}",
                            f"{pb.recx[k]:.4f}", "0.0000", ev, f"{pb.srcy[s]:.4f}",
                            f"{pb.srcx[s]:.4f}", "0.0000", f"{pb.periods[pb.pidx[s]]:.4f}",
                            f"{pb.weight[k]:.4f}", f"{dist:.4f}",
                            f"{dist / tt[pb.path[k]]:.6f}"])


def read_src_rec_tt(fname):
    with open(fname) as f:
        r = csv.DictReader(f)
        return np.array([float(row["tt"]) for row in r])


# ---------------------------------------------------------------------------
# 3-D kernel combination and multigrid projection inputs
# ---------------------------------------------------------------------------
def linspace_ref(first: float, last: float, n: int) -> np.ndarray:
    """linspace_r8r8 (src/shared/utils.f90:592-604): first + step*(i-1),
    last node set to `last`."""
    step = (last - first) / (n - 1)
    v = first + step * np.arange(n, dtype=np.float64)
    v[-1] = last
    return v


def inv_grids(xgrids, ygrids, zgrids, n_inv_grid, nset):
    """get_inv_grids (src/model.f90:127-172): the nset shifted inversion
    grids, (xinv, yinv, zinv), each (ninv, nset) in Fortran order."""
    nix, niy, niz = (int(v) for v in n_inv_grid)
    x1, xn = float(xgrids[0]), float(xgrids[-1])
    y1, yn = float(ygrids[0]), float(ygrids[-1])
    z1, zn = float(zgrids[0]), float(zgrids[-1])
    ix = linspace_ref(x1 - (xn - x1) / (nix - 2) / 2.0, xn + (xn - x1) / (nix - 2) / 2.0, nix)
    iy = linspace_ref(y1 - (yn - y1) / (niy - 2), yn, niy)
    iz = linspace_ref(z1 - 0.5 * (zn - z1) / (niz - 2), zn + 0.5 * (zn - z1) / (niz - 2), niz)
    zref = np.concatenate([iz[1:], iz[-1:]])
    zadd = (zref - iz) / (nset + 1)
    zadd[0] = 0
    xinv = np.zeros((nix, nset), order="F")
    yinv = np.zeros((niy, nset), order="F")
    zinv = np.zeros((niz, nset), order="F")
    polar = 1
    for i in range(nset):
        if i == 0:
            xinv[:, 0] = ix
        else:
            xinv[:, i] = xinv[:, i - 1] + polar * i * (ix[1] - ix[0]) / (nset + 1)
            polar = -polar
        yinv[:, i] = iy + i * (iy[1] - iy[0]) / (nset + 1)
        zinv[:, i] = iz + i * zadd
    return xinv, yinv, zinv


def brocher_vp(vs):
    """Brocher (2005) Vp from Vs (km/s), the relation behind the reference's
    empirical_vp / dalpha_dbeta."""
    vs = np.asarray(vs, np.float64)
    return 0.9409 + 2.0947 * vs - 0.8206 * vs ** 2 + 0.2683 * vs ** 3 - 0.0251 * vs ** 4


@dataclasses.dataclass
class Kernel3D:
    """Inputs of combine_kernels + post_processing_for_kernel for one data
    type, in the reference's layouts (Fortran order): adj_s / adj_density
    (P, nx, ny), sen_vs / sen_vp / sen_rho (P, nx, ny, nz), vs3d / vp3d
    (nx, ny, nz), model axes, inversion grids (ninv, nset)."""
    name: str
    xgrids: np.ndarray
    ygrids: np.ndarray
    zgrids: np.ndarray
    adj_s: np.ndarray
    adj_density: np.ndarray
    sen_vs: np.ndarray
    sen_vp: np.ndarray
    sen_rho: np.ndarray
    vs3d: np.ndarray
    vp3d: np.ndarray
    xinv: np.ndarray
    yinv: np.ndarray
    zinv: np.ndarray
    periods: np.ndarray
    chi0: float = 1.0
    weight: float = 1.0

    @property
    def shape(self):
        return self.sen_vs.shape


def kernel3d_case(nx=60, ny=60, nz=30, nperiod=16, d=0.1, zmax=60.0, n_inv_grid=(8, 9, 8),
                  nset=5, seed=2, adj_s=None, adj_density=None, name=None):
    """Config 2's model (60 x 60 x 30 nodes, 0.1 deg, 0-60 km, Vs linear
    3.2 -> 4.5 km/s with a +-5 % 2x3x2 checkerboard, 16 periods 2-40 s) with
    the first example's inversion grids (ncomponents 5, n_inv_grid 8 x 9 x 8).
    The depth sensitivity kernels come from surfdisp96 in the reference
    (out of scope): seeded stand-ins here, a depth bump per period centred
    near a third of the wavelength, modulated laterally.  adj_s /
    adj_density: (P, nx, ny) fields (e.g. an engine evaluation on the model
    grid, transposed), else seeded smooth fields of both signs."""
    rng = np.random.default_rng(seed)
    xg, yg = arange_grid(100.0, nx, d), arange_grid(22.0, ny, d)
    zg = np.linspace(0.0, zmax, nz)
    periods = np.geomspace(2.0, 40.0, nperiod)
    cbxy = checkerboard_2d(nx, ny, 2, 3, 1.0) - 1.0
    cbz = np.sin(2 * PI_F * np.arange(1, nz + 1) / nz)
    vs = (3.2 + 1.3 * zg / zmax)[None, None, :] * (1 + 0.05 * cbxy[:, :, None] * cbz[None, None, :])
    vs = np.asfortranarray(vs)
    vp = np.asfortranarray(brocher_vp(vs))
    X = np.linspace(0, 1, nx)[:, None]
    Y = np.linspace(0, 1, ny)[None, :]
    if adj_s is None:
        ph = rng.uniform(0, 2 * np.pi, (nperiod, 2))
        adj_s = np.stack([1e-3 * np.sin(3 * X + ph[p, 0]) * np.cos(2 * Y + ph[p, 1])
                          for p in range(nperiod)])
    if adj_density is None:
        adj_density = np.abs(adj_s) * (1 + 0.1 * rng.random(adj_s.shape))
    sen = []
    for k in range(3):
        s = np.zeros((nperiod, nx, ny, nz))
        for p, T in enumerate(periods):
            zc = 3.5 * T / 3.0
            w = max(0.25 * 3.5 * T, 2 * (zg[1] - zg[0]))
            bump = np.exp(-((zg - zc) / w) ** 2) * (0.5 - 0.2 * k)
            lat = 1 + 0.05 * np.cos(2 * np.pi * (X + 0.3 * k)) * np.sin(2 * np.pi * Y)
            s[p] = lat[:, :, None] * bump[None, None, :]
        sen.append(np.asfortranarray(s))
    xinv, yinv, zinv = inv_grids(xg, yg, zg, n_inv_grid, nset)
    return Kernel3D(name=name or f"kernel3d_{nx}x{ny}x{nz}_{nperiod}per", xgrids=xg, ygrids=yg,
                    zgrids=zg, adj_s=np.asfortranarray(adj_s),
                    adj_density=np.asfortranarray(adj_density), sen_vs=sen[0], sen_vp=sen[1],
                    sen_rho=sen[2], vs3d=vs, vp3d=vp, xinv=xinv, yinv=yinv, zinv=zinv,
                    periods=periods, chi0=float(np.sum(np.abs(adj_s))) + 1.0, weight=1.0)


# ---------------------------------------------------------------------------
# src_rec tables
# ---------------------------------------------------------------------------
def srcrec_rows_all_pairs(sx, sy, periods, tt_fn, names=None, weight=1.0):
    """Rows of a src_rec table (dicts with the CSV's columns) where every
    station is an event and every other station its receiver, for every
    period: grouped by event, then period, then station, as the reference's
    example tables are.  tt_fn(p, e, r) gives the time."""
    n = len(sx)
    names = names or [f"ST{i:04d}" for i in range(n)]
    rows = []
    for e in range(n):
        for p, T in enumerate(periods):
            for r in range(n):
                if r == e:
                    continue
                rows.append(dict(tt=float(tt_fn(p, e, r)), staname=names[r], stla=float(sy[r]),
                                 stlo=float(sx[r]), evtname=names[e], evla=float(sy[e]),
                                 evlo=float(sx[e]), period=float(T), weight=float(weight)))
    return rows


def config2_srcrec_rows(nsta=80, nperiod=16, seed=1):
    """Config 2's acquisition as a src_rec table: 80 stations, each an
    event with the other 79 as receivers, 16 periods (101,120 paths);
    times are great-circle distance over 3.5 km/s with 3 % seeded noise."""
    rng = np.random.default_rng(seed)
    xx, yy = arange_grid(100.0, 120, 0.05), arange_grid(22.0, 120, 0.05)
    sx, sy = _stations(rng, nsta, xx[0], xx[-1], yy[0], yy[-1])
    periods = np.geomspace(2.0, 40.0, nperiod)
    dist = gps2dist(sy[:, None], sx[:, None], sy[None, :], sx[None, :])
    noise = rng.normal(0, 0.03, (nperiod, nsta, nsta))
    return srcrec_rows_all_pairs(sx, sy, periods,
                                 lambda p, e, r: dist[e, r] / 3.5 * (1 + noise[p, e, r]))
