"""The entry point that allocates nothing (surfatt_uw_lonlat_solve_noalloc).

It exists for callers that must not allocate device memory when they call the
solver -- e.g. a host framework whose memory pool owns the GPU's memory, or a
loop that cannot afford the device-wide synchronisation of cudaMalloc and
cudaFree.  It takes device arrays and uses a fixed scratch array compiled into
the library.  This test calls it through the C ABI twice in a row, the second
time on a smaller grid with another source (so the scratch regions sit at
other offsets and hold other sizes: leftovers of the first call would show),
and compares each result with the ordinary drop-in entry point,
fsm_uw_ps_lonlat_2d_ (the same FP64 solver code on the same inputs; the
per-grid metric is precomputed by a different kernel, so the two may differ
in the last bits: 1e-10 relative), and with the oracle within the plain
path's travel-time tolerance (1e-6).  The file is
collected last so that a run stopping at the first failure has already run
every other test.
"""
import numpy as np
import pytest

from conftest import rel_pointwise
from surfatt_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TT_TOL = 1e-6
SAME_SOLVER_TOL = 1e-10


def _case(nx, ny, m12):
    xx, yy = W.arange_grid(100.0, nx, 0.05), W.arange_grid(22.0, ny, 0.05)
    m11 = np.ones((nx, ny))
    m22 = np.ones((nx, ny))
    m12 = np.full((nx, ny), m12)
    fun = 1.0 / (3.0 * W.checkerboard_2d(nx, ny, 2, 3, 0.06))
    return xx, yy, m11, m22, m12, fun


def test_noalloc_matches_dropin_two_calls(sg, oracle):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev).cuda_stream
    col = lambda a: torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).to(dev)
    # first call: 120 x 110 (13200 cells); second: 70 x 53 with another source
    for (nx, ny, m12, src) in ((120, 110, 0.02, (101.03, 23.01)),
                               (70, 53, -0.03, (102.61, 23.77))):
        xx, yy, m11, m22, m12a, fun = _case(nx, ny, m12)
        d_xx, d_yy = torch.from_numpy(xx).to(dev), torch.from_numpy(yy).to(dev)
        d_a, d_b, d_c, d_f = col(m11), col(m22), col(-m12a), col(fun)
        d_T = torch.full((nx * ny,), -1.0, dtype=torch.float64, device=dev)
        d_si = torch.full((2,), -7, dtype=torch.int32, device=dev)
        st = sg.uw_lonlat_solve_noalloc(d_xx.data_ptr(), d_yy.data_ptr(), nx, ny, d_a.data_ptr(),
                                        d_b.data_ptr(), d_c.data_ptr(), d_f.data_ptr(), *src,
                                        d_T.data_ptr(), d_si.data_ptr(), stream)
        assert st == sg.OK
        torch.cuda.synchronize(dev)
        T = d_T.cpu().numpy().reshape((nx, ny), order="F")
        status, iters = (int(v) for v in d_si.cpu().numpy())
        Td, sd, idr = sg.fsm_uw_ps_lonlat_2d(xx, yy, m11, m22, -m12a, fun, *src)
        assert status == sd == sg.OK
        assert iters == idr
        assert rel_pointwise(T, Td) <= SAME_SOLVER_TOL
        Tr, sr, ir = oracle.fsm_uw_ps_lonlat_2d(xx, yy, m11, m22, -m12a, fun, *src)
        assert sr == 0 and iters == ir
        assert rel_pointwise(T, Tr) <= TT_TOL


def test_noalloc_rejects_oversize_grid(sg):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    z = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    st = sg.uw_lonlat_solve_noalloc(z.data_ptr(), z.data_ptr(), 200, 200, z.data_ptr(),
                                    z.data_ptr(), z.data_ptr(), z.data_ptr(), 0.0, 0.0,
                                    z.data_ptr(), z.data_ptr(), 0)
    assert st == sg.BAD_ARG
