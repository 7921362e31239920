import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "surfatt-iso_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def sg():
    import surfatt_gb300
    surfatt_gb300.build()
    surfatt_gb300.lib()
    return surfatt_gb300


def rel_max(a, b):
    """max |a-b| / max |b| (norm-wise relative error of a field)."""
    import numpy as np
    den = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / (den if den > 0 else 1.0)


def rel_pointwise(a, b):
    """max |a-b|/|b| over entries with b != 0 (travel times)."""
    import numpy as np
    m = b != 0
    return float(np.max(np.abs(a[m] - b[m]) / np.abs(b[m]))) if m.any() else 0.0
