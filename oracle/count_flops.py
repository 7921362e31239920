"""Floating-point operations per sweep visit of the reference formulation.

Runs a sample of a workload through the counting build of the oracle
(libsurfatt_oracle_count.so, -DORC_COUNT_FLOPS) and converts the case tallies
into flops per visit, counting add/sub/mul/div/sqrt as one flop each, as
FSM_UW_PS_lonlat_2d and FSM_O1_JSE_lonlat_2d write them
(src/eikon_solver_2d.f90):

  two-sided case (:911-994)        44 flops (px, qx, py, qy, eqn_a/b/c, Delta)
    + when Delta >= 0              28 flops (two roots, Tx, Ty, characteristics)
  one-sided case (:996-1075)       21 flops (px, qx, dis, two roots and tests)
  adjoint visit (:1392-1402)       16 flops (d, e, (delta+e)/d)

Usage (from the repository root):
  python oracle/count_flops.py config2 32
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TWO_SIDED, DELTA_BRANCH, ONE_SIDED, ADJ_VISIT = 44, 28, 21, 16


def count(pb, solves, mode=3):
    import oracle as O
    O.build()
    lib = ctypes.CDLL(os.path.join(HERE, "_build", "libsurfatt_oracle_count.so"))
    sub = pb.subset(solves)
    saved = O._lib
    O._lib = None
    O._LIB_PATH_SAVED = O._LIB_PATH
    O._LIB_PATH = os.path.join(HERE, "_build", "libsurfatt_oracle_count.so")
    try:
        r = O.gradient_eval(sub, mode=mode, nthreads=1)
        c = (ctypes.c_longlong * 5)()
        O.lib().orc_flop_counts(c)
    finally:
        O._LIB_PATH = O._LIB_PATH_SAVED
        O._lib = saved
    visits, two, delta, one, adj = list(c)
    fwd = (TWO_SIDED * two + DELTA_BRANCH * delta + ONE_SIDED * one) / max(visits, 1)
    return dict(fwd_visits=visits, adj_visits=adj, fwd_flops_per_visit=fwd,
                adj_flops_per_visit=float(ADJ_VISIT), delta_fraction=delta / max(two, 1),
                fwd_iters=r["fwd_iters"].tolist(), adj_iters=r["adj_iters"].tolist())


def main():
    sys.path.insert(0, HERE)
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "surfatt-iso_gb300"))
    from surfatt_gb300 import workloads as W
    name = sys.argv[1] if len(sys.argv) > 1 else "config2"
    nsample = int(sys.argv[2]) if len(sys.argv) > 2 else 32
    pb = getattr(W, name)()
    per = max(1, nsample // pb.nperiod)
    solves = []
    for p in range(pb.nperiod):
        idx = np.nonzero(pb.pidx == p)[0]
        solves += list(idx[:per])
    res = count(pb, solves[:nsample], mode=pb.mode)
    for k, v in res.items():
        if not isinstance(v, list):
            print(f"{k}: {v}")


if __name__ == "__main__":
    main()
