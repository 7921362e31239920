"""Generate the committed golden fixtures with the CPU oracle.

  config1_src_rec.csv  config 1's 600 paths in the reference's src_rec CSV
                       layout (src/src_rec.f90:285-325); `tt` = forward times
                       of the +-6 % 2x3 checkerboard model (the "observed"
                       data), F0.6 like the reference's writer.
  small_cases.npz      inputs and oracle outputs of small solves (forward
                       lon/lat, adjoint, mask, interp2, one 3-D gradient
                       evaluation) used by the CPU suite to detect any change
                       of the oracle and by the GPU suite as a second check.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "surfatt-iso_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from surfatt_gb300 import workloads as W  # noqa: E402


def config1_csv():
    true = W.config1_true_model()
    r = O.gradient_eval(true, mode=0, nthreads=4)
    assert r["rc"] == 0
    pb = W.config1()
    W.write_src_rec_csv(os.path.join(HERE, "config1_src_rec.csv"), pb, tt=r["tt_fwd"])


def small_cases():
    out = {}
    nx, ny = 23, 19
    xx, yy = W.arange_grid(100.0, nx, 0.05), W.arange_grid(22.0, ny, 0.05)
    one = np.ones((nx, ny))
    sv = 3.0 * W.checkerboard_2d(nx, ny, 2, 3, 0.06)
    fun = 1.0 / sv
    T, st, it = O.fsm_uw_ps_lonlat_2d(xx, yy, one, one, 0 * one, fun, 100.53, 22.47)
    out.update(fw_xx=xx, fw_yy=yy, fw_fun=fun, fw_src=np.array([100.53, 22.47]), fw_T=T,
               fw_iters=np.array([it]))
    xr = np.array([100.13, 100.91, 100.42, 100.77])
    yr = np.array([22.12, 22.21, 22.79, 22.66])
    sadj = np.array([0.7, -1.2, 0.4, 2.0])
    Ta, st2, it2 = O.fsm_o1_jse_lonlat_2d(xx, yy, one, one, 0 * one, T, xr, yr, sadj)
    out.update(adj_xr=xr, adj_yr=yr, adj_s=sadj, adj_Ta=Ta, adj_iters=np.array([it2]))
    out.update(mask_T=O.mask(xx, yy, Ta, 100.53, 22.47))
    out.update(interp=np.array([O.interp2(xx, yy, T, x, y) for x, y in zip(xr, yr)]))
    pb = W.flat_case(nx=27, ny=25, nsta=4, nperiod=2, mode=3)
    g = O.gradient_eval(pb, mode=3, nthreads=1)
    out.update(ge_adj_s=g["adj_s"], ge_adj_density=g["adj_density"], ge_chi=np.array([g["chi"]]),
               ge_tt=g["tt_fwd"], ge_fwd_iters=g["fwd_iters"], ge_adj_iters=g["adj_iters"])
    np.savez_compressed(os.path.join(HERE, "small_cases.npz"), **out)


if __name__ == "__main__":
    config1_csv()
    small_cases()
    print("golden fixtures written to", HERE)
