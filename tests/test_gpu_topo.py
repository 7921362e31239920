"""Surface metric from topography on the GPU vs the oracle (GPU only).
The smoothing differs from the reference's evaluation by rounding (see
test_gpu_smooth), the gradient and metric are explicitly rounded as
written, the dip angle uses the device's atan: norm-wise 1e-12."""
import numpy as np
import pytest

from conftest import rel_max
from surfatt_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.mark.parametrize("shape,d,sigmas", [((60, 50), 0.02, [0.03, 0.06, 0.1]),
                                            ((150, 200), 0.02, [0.04]),
                                            ((33, 17), 0.05, [0.2, 0.5])])
def test_topo_metric_matches_oracle(sg, oracle, shape, d, sigmas):
    xx, yy, topo, *_ = W.config5_model(n_lon=shape[0], n_lat=shape[1], d=d)
    got = sg.topo_metric(topo, xx, yy, sigmas)
    ref = oracle.topo_metric(topo, xx, yy, sigmas)
    for g, r in zip(got, ref):
        assert g.shape == r.shape
        for p in range(len(sigmas)):
            assert rel_max(g[p], r[p]) <= TOL
    ms, n = sg.topo_metric_timing()
    assert ms > 0 and n == 3


def test_topo_sigma_formula(sg):
    v, T = np.array([3.1, 3.4]), np.array([10.0, 20.0])
    pi_s = float(np.float32(3.14159265359))
    km2deg = 1.0 / (6371.0 * pi_s / 180.0)
    assert np.array_equal(sg.topo_sigma(v, T, 0.5), v * T * 0.5 * km2deg / (2.0 * pi_s))
