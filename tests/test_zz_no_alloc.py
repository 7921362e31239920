"""The entry point that allocates nothing (surfatt_uw_lonlat_solve_noalloc).

It exists for callers that must not allocate device memory when they call the
solver -- e.g. a host framework whose memory pool owns the GPU's memory, or a
loop that cannot afford the device-wide synchronisation of cudaMalloc and
cudaFree.  It takes device arrays and uses a fixed scratch array compiled into
the library.  This test calls it through the C ABI twice in a row (different
sources, so stale scratch from the first call would show) and compares each
result with the ordinary drop-in entry point, fsm_uw_ps_lonlat_2d_.  The file
is collected last so that a run stopping at the first failure has already run
every other test.
"""
import numpy as np
import pytest

from conftest import rel_pointwise
from surfatt_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TT_TOL = 1e-6


def test_noalloc_matches_dropin_two_calls(sg):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    nx, ny = 120, 110
    xx, yy = W.arange_grid(100.0, nx, 0.05), W.arange_grid(22.0, ny, 0.05)
    m11 = np.ones((nx, ny))
    m22 = np.ones((nx, ny))
    m12 = np.full((nx, ny), 0.02)
    fun = 1.0 / (3.0 * W.checkerboard_2d(nx, ny, 2, 3, 0.06))
    dev = torch.device("cuda:0")
    col = lambda a: torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).to(dev)
    d_xx, d_yy = torch.from_numpy(xx).to(dev), torch.from_numpy(yy).to(dev)
    d_a, d_b, d_c, d_f = col(m11), col(m22), col(-m12), col(fun)
    d_T = torch.zeros(nx * ny, dtype=torch.float64, device=dev)
    d_si = torch.zeros(2, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for src in ((101.03, 23.01), (104.77, 26.02)):
        d_T.fill_(-1.0)
        st = sg.uw_lonlat_solve_noalloc(d_xx.data_ptr(), d_yy.data_ptr(), nx, ny, d_a.data_ptr(),
                                        d_b.data_ptr(), d_c.data_ptr(), d_f.data_ptr(), *src,
                                        d_T.data_ptr(), d_si.data_ptr(), stream)
        assert st == sg.OK
        torch.cuda.synchronize(dev)
        T = d_T.cpu().numpy().reshape((nx, ny), order="F")
        status, iters = (int(v) for v in d_si.cpu().numpy())
        Tr, sr, ir = sg.fsm_uw_ps_lonlat_2d(xx, yy, m11, m22, -m12, fun, *src)
        assert status == sr == sg.OK
        assert iters == ir
        assert rel_pointwise(T, Tr) <= TT_TOL


def test_noalloc_rejects_oversize_grid(sg):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    z = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    st = sg.uw_lonlat_solve_noalloc(z.data_ptr(), z.data_ptr(), 200, 200, z.data_ptr(),
                                    z.data_ptr(), z.data_ptr(), z.data_ptr(), 0.0, 0.0,
                                    z.data_ptr(), z.data_ptr(), 0)
    assert st == sg.BAD_ARG
