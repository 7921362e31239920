"""The GPU-built work list of a src_rec table vs the oracle's string scans
(GPU only): solves, sources and receiver gathers equal exactly."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from surfatt_gb300 import workloads as W
from test_srcrec import _oracle_rows, _read_py, tricky_rows

pytestmark = pytest.mark.gpu

KEYS_SOLVE = ("pidx", "sta", "srcx", "srcy", "rec_off", "nrec")
KEYS_REC = ("recx", "recy", "tt", "weight", "path")


def _table(sg, rows):
    return sg.SrcRec.from_arrays(*[[r[k] for r in rows] for k in
                                   ("evtname", "staname", "stla", "stlo", "evla", "evlo",
                                    "period", "tt")], weight=[r["weight"] for r in rows])


def _check(sg, oracle, rows):
    t = _table(sg, rows)
    ns = t.build_worklist(0)
    wl = t.worklist()
    o = _oracle_rows(oracle, rows)
    assert ns == len(o["pidx"])
    for k in KEYS_SOLVE:
        assert np.array_equal(wl[k], o[k]), k
    nr = int(o["nrec"].sum())
    for k in KEYS_REC:
        assert np.array_equal(wl[k], o[k][:nr]), k
    ms, n = t.build_timing()
    assert ms > 0 and n == 5
    t.close()


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_worklist_tricky_tables(sg, oracle, seed):
    _check(sg, oracle, tricky_rows(seed))


def test_worklist_shuffled_large(sg, oracle):
    rows = W.config2_srcrec_rows(nsta=30, nperiod=12, seed=5)
    rng = np.random.default_rng(6)
    rows = [rows[i] for i in rng.permutation(len(rows))]
    _check(sg, oracle, rows)


def test_worklist_config1_fixture(sg, oracle):
    _check(sg, oracle, _read_py(os.path.join(GOLDEN, "config1_src_rec.csv")))


def test_engine_from_table_matches_oracle(sg, oracle):
    """config 1's src_rec fixture -> table -> GPU work list -> engine: the
    gradient evaluation of the assembled problem matches the oracle's on
    the same problem (plain FP64 bars), and its synthetic-time table has one
    entry per CSV row."""
    from conftest import rel_max, rel_pointwise
    fn = os.path.join(GOLDEN, "config1_src_rec.csv")
    pb = W.config1(observed_tt=W.read_src_rec_tt(fn))
    t = sg.SrcRec.read_csv(fn)
    t.build_worklist(0)
    grids = [pb.grid(0)]
    fields = [dict(svel=pb.field("svel", 0), m11=pb.field("m11", 0), m12=pb.field("m12", 0),
                   m22=pb.field("m22", 0))]
    pt = t.problem(grids, fields, mode=2)
    assert pt.nsolve == 25 and pt.npath == 600
    eng = sg.Engine(0)
    got = eng.evaluate(pt, mode=2, precision=sg.PREC_FP64)
    ref = oracle.gradient_eval(pt, mode=2, nthreads=8)
    assert rel_pointwise(got["tt_fwd"], ref["tt_fwd"]) <= 1e-6
    assert rel_max(got["adj_s"], ref["adj_s"]) <= 1e-5
    assert abs(got["chi"] - ref["chi"]) <= 1e-6 * abs(ref["chi"])
    eng.close()
    t.close()
