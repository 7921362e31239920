"""Serving workload on a curved surface and a Poisson request driver.

The surface: a seeded Gaussian island (peak 4 km, radius 40 km) plus 200 m
random-field roughness (workloads.config5_model), whose surface metric
(src/grid.f90:117-145) is resampled onto lon/lat grids of several sizes
(64^2 .. 512^2 nodes) covering the island.  A request is one of
  * a gradient evaluation (3-D mode: two adjoints per solve),
  * a line-search trial (forward only, perturbed velocity model),
  * a forward-only checkerboard run (forward only, checkerboard model)
over 10-120 sources and 1-15 periods of one grid.  Station tables (work
lists) and the per-grid metric stay resident in the server; trial and
checkerboard velocities travel with their requests.
"""
import math
import threading
import time

import numpy as np

from . import workloads as W


def _resample(field, xx0, yy0, xx, yy):
    """Bilinear resampling of a (len(xx0), len(yy0)) field onto (xx, yy)."""
    fx = np.interp(xx, xx0, np.arange(len(xx0)))
    fy = np.interp(yy, yy0, np.arange(len(yy0)))
    i0 = np.clip(np.floor(fx).astype(int), 0, len(xx0) - 2)
    j0 = np.clip(np.floor(fy).astype(int), 0, len(yy0) - 2)
    tx = (fx - i0)[:, None]
    ty = (fy - j0)[None, :]
    I, J = i0[:, None], j0[None, :]
    return ((1 - tx) * (1 - ty) * field[I, J] + tx * (1 - ty) * field[I + 1, J] +
            (1 - tx) * ty * field[I, J + 1] + tx * ty * field[I + 1, J + 1])


class Catalog:
    """Grids, per-period velocity models and station tables of the serving run."""

    def __init__(self, sides=(64, 96, 128, 192, 256, 384, 512), nperiod=15, nsta=140, seed=4):
        rng = np.random.default_rng(seed)
        xx0, yy0, topo, m11, m12, m22 = W.config5_model(seed=seed)
        self.periods = np.geomspace(3.0, 30.0, nperiod)
        lo_x, hi_x = xx0[0] + 0.1, xx0[-1] - 0.1
        lo_y, hi_y = yy0[0] + 0.1, yy0[-1] - 0.1
        self.stx, self.sty = W._stations(rng, nsta, lo_x, hi_x, lo_y, hi_y, frac=0.85)
        self.models = {}
        for n in sides:
            xx = W.arange_grid(lo_x, n, (hi_x - lo_x) / (n - 1))
            yy = W.arange_grid(lo_y, n, (hi_y - lo_y) / (n - 1))
            a = _resample(m11, xx0, yy0, xx, yy)
            c = _resample(m12, xx0, yy0, xx, yy)
            b = _resample(m22, xx0, yy0, xx, yy)
            grids, fields = [], []
            km = W.R_EARTH * math.pi / 180
            for p, T in enumerate(self.periods):
                grf = W.gaussian_random_field(rng, n, n, (xx[1] - xx[0]) * km,
                                              (yy[1] - yy[0]) * km, 25.0, 0.03)
                sv = (3.0 + 0.03 * T) * (1 + grf)
                grids.append((xx, yy))
                fields.append(dict(svel=sv, m11=a, m12=c, m22=b))
            self.models[n] = W._pack(f"surface_{n}", grids, fields,
                                     [(0, xx[n // 2], yy[n // 2], xx[:1] + 0.01, yy[:1] + 0.01,
                                       np.ones(1), np.ones(1))], self.periods, 3)

    def worklist(self, n, sources, periods, mode, seed):
        """Sources x periods of grid n; receivers: the other stations."""
        rng = np.random.default_rng(seed)
        base = self.models[n]
        sx, sy = self.stx, self.sty
        solves = []
        for p in periods:
            for s in sources:
                r = np.array([k for k in range(len(sx)) if k != s])
                d = W.gps2dist(sy[s], sx[s], sy[r], sx[r])
                tt = d / (3.0 + 0.03 * self.periods[p]) * (1 + rng.normal(0, 0.02, len(r)))
                solves.append((int(p), sx[s], sy[s], sx[r], sy[r], tt, np.ones(len(r))))
        pb = W.Problem(**{f: getattr(base, f) for f in (
            "name", "nperiod", "nx", "ny", "xoff", "yoff", "goff", "xgrid", "ygrid", "svel", "m11",
            "m12", "m22", "periods")},
            pidx=np.array([s[0] for s in solves], np.int32),
            srcx=np.array([s[1] for s in solves]), srcy=np.array([s[2] for s in solves]),
            rec_off=np.concatenate([[0], np.cumsum([len(s[3]) for s in solves])[:-1]]).astype(np.int32),
            nrec=np.array([len(s[3]) for s in solves], np.int32),
            recx=np.concatenate([s[3] for s in solves]), recy=np.concatenate([s[4] for s in solves]),
            tt=np.concatenate([s[5] for s in solves]), weight=np.concatenate([s[6] for s in solves]),
            path=np.arange(sum(len(s[3]) for s in solves), dtype=np.int32), mode=mode)
        return pb


def make_requests(cat, count, seed=4, max_solves=600, grid_weights=None):
    """Request list: (grid n, worklist problem, kind, velocity override or None)."""
    rng = np.random.default_rng(seed + 1000)
    sides = sorted(cat.models)
    w = np.asarray(grid_weights if grid_weights is not None
                   else [1.0 / (s / sides[0]) ** 1.5 for s in sides])
    w = w / w.sum()
    out = []
    for q in range(count):
        n = int(rng.choice(sides, p=w))
        nsrc = int(rng.integers(10, 121))
        nper = int(rng.integers(1, 16))
        while nsrc * nper > max_solves:
            nper = max(1, nper // 2)
            if nsrc * nper > max_solves:
                nsrc = max(10, nsrc // 2)
        src = np.sort(rng.choice(len(cat.stx), nsrc, replace=False))
        per = np.sort(rng.choice(len(cat.periods), nper, replace=False))
        kind = rng.choice(["gradient", "linesearch", "checkerboard"], p=[0.5, 0.3, 0.2])
        mode = 3 if kind == "gradient" else 0
        pb = cat.worklist(n, src, per, mode, seed=seed * 7919 + q)
        vel = None
        if kind == "linesearch":
            vel = pb.svel * (1 + 0.01 * rng.normal())
        elif kind == "checkerboard":
            cb = np.concatenate([W.checkerboard_2d(int(pb.nx[p]), int(pb.ny[p]), 3, 3, 0.05)
                                 .ravel(order="F") for p in range(pb.nperiod)])
            vel = pb.svel * cb
        out.append(dict(n=n, pb=pb, kind=str(kind), mode=mode, vel=vel, nsolve=pb.nsolve))
    return out


def run_poisson(server, requests, rate_per_s, precision, seed=4, model_ids=None):
    """Submit the requests at Poisson arrival times (mean rate `rate_per_s`)
    from one thread and collect them from another.  Returns per-request
    latencies (ms), statuses, the wall time and the solves completed."""
    rng = np.random.default_rng(seed + 2000)
    gaps = rng.exponential(1.0 / rate_per_s, len(requests))
    wls = [server.add_worklist(model_ids[r["n"]], r["pb"]) for r in requests]
    tickets = [None] * len(requests)
    ready = [threading.Event() for _ in requests]
    lat = [0.0] * len(requests)
    sts = [None] * len(requests)

    def waiter():
        for q in range(len(requests)):
            ready[q].wait()
            st, _, ms = server.wait(tickets[q])
            sts[q] = st
            lat[q] = ms

    th = threading.Thread(target=waiter)
    th.start()
    server.reset_stats()
    t0 = time.perf_counter()
    for q, r in enumerate(requests):
        target = t0 + float(np.sum(gaps[:q + 1]))
        now = time.perf_counter()
        if target > now:
            time.sleep(target - now)
        tickets[q] = server.submit(wls[q], r["vel"], r["mode"], precision)
        ready[q].set()
    th.join()
    wall = time.perf_counter() - t0
    return dict(latency_ms=lat, status=sts, wall_s=wall,
                solves=int(sum(r["nsolve"] for r in requests)))
