"""Pins of the oracle's topography metric (no GPU): gradient_2_geo of a
field linear in longitude or latitude against its analytic derivative,
a flat topography's metric, and the metric identities."""
import math

import numpy as np
import pytest

from surfatt_gb300 import workloads as W

R = 6371.0
D2R = float(np.float32(3.14159265359)) / 180.0


def test_gradient_of_linear_fields(oracle):
    lon, lat = W.arange_grid(100.0, 30, 0.05), W.arange_grid(22.0, 20, 0.05)
    fx_true = 0.7 / (R * D2R * np.cos(np.radians(lat)))
    tx, ty = oracle.gradient_2_geo(0.7 * lon[:, None] + 0 * lat[None, :], lon, lat)
    assert np.max(np.abs(tx / fx_true[None, :] - 1)) <= 1e-12 and np.max(np.abs(ty)) == 0
    tx, ty = oracle.gradient_2_geo(0 * lon[:, None] - 1.3 * lat[None, :], lon, lat)
    assert np.max(np.abs(ty / (-1.3 / (R * D2R)) - 1)) <= 1e-12 and np.max(np.abs(tx)) == 0


def test_flat_topography(oracle):
    lon, lat = W.arange_grid(100.0, 25, 0.02), W.arange_grid(22.0, 21, 0.02)
    m11, m22, m12, ang = oracle.topo_metric(np.full((25, 21), 1.5), lon, lat, [0.03, 0.05])
    # the smoothed field is 1.5 to rounding, so its gradient is at rounding level
    assert np.max(np.abs(m11 - 1)) <= 1e-15 and np.max(np.abs(m22 - 1)) <= 1e-15
    assert np.max(np.abs(m12)) <= 1e-30 and np.max(ang) <= 1e-12


def test_metric_identities(oracle):
    xx, yy, topo, *_ = W.config5_model(n_lon=40, n_lat=36, d=0.02)
    m11, m22, m12, ang = oracle.topo_metric(topo, xx, yy, [0.04, 0.08])
    # a, b, c of a unit normal: a + b = 1 + 1/(1+|g|^2), a*b - c^2 = 1/(1+|g|^2)
    g2 = np.tan(np.radians(ang)) ** 2
    assert np.max(np.abs(m11 + m22 - (1 + 1 / (1 + g2)))) <= 1e-12
    assert np.max(np.abs(m11 * m22 - m12 ** 2 - 1 / (1 + g2))) <= 1e-12
    assert np.all(ang[1] <= ang[0].max() + 1e-12)    # more smoothing, gentler slopes
