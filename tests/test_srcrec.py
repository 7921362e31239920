"""The src_rec table (no GPU): CSV reading / writing of the native library,
and pins of the oracle's work list against a second restatement.

The reference has no tests for these routines; the oracle
(oracle/oracle_srcrec.c) is pinned against the pure-Python restatement
below on tables built to exercise every rule (shuffled rows, an event that
is not a station, a station whose coordinates differ between rows, names
with trailing blanks, a period of exactly 0, weights), and the native CSV
reader against Python's csv module on the committed fixture and, where the
reference checkout is present, on its example tables.
"""
import csv
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN

EXAMPLES = "/root/reference/examples"


def py_worklist(rows):
    """Literal restatement of get_periods, get_sta, scatter_src_gather,
    get_periods_by_src, get_evt_gather, get_sta_pos (src/src_rec.f90)."""
    name = lambda s: s.rstrip(" ")
    periods = []
    for r in rows:
        if not any(p == r["period"] for p in periods):
            periods.append(r["period"])
    periods.sort()
    sta, lo, la = [], [], []
    for r in rows:
        if name(r["staname"]) not in sta:
            sta.append(name(r["staname"]))
            la.append(r["stla"])
            lo.append(r["stlo"])
    for r in rows:
        if name(r["evtname"]) not in sta:
            sta.append(name(r["evtname"]))
            la.append(r["evla"])
            lo.append(r["evlo"])
    out = dict(periods=periods, sta=sta, lo=lo, la=la, solves=[])
    for j, sname in enumerate(sta):
        if not any(name(r["evtname"]) == sname for r in rows):
            continue
        stp = [0.0] * len(periods)
        n = 0
        for r in rows:
            if name(r["evtname"]) != sname or any(v == r["period"] for v in stp):
                continue
            stp[n] = r["period"]
            n += 1
            ip = periods.index(r["period"])
            recs = []
            for m, q in enumerate(rows):
                if name(q["evtname"]) == sname and q["period"] == periods[ip]:
                    k = max(i for i, s2 in enumerate(sta) if s2 == name(q["staname"]))
                    recs.append((lo[k], la[k], q["tt"], q.get("weight", 1.0), m))
            k = sta.index(sname)
            out["solves"].append((ip, j, lo[k], la[k], recs))
    return out


def tricky_rows(seed=0, nsta=9, nper=5, npath=300):
    rng = np.random.default_rng(seed)
    per = [5.0, 2.5, 10.0, 0.0, 7.5][:nper]
    names = [f"S{i:02d}" for i in range(nsta)]
    rows = []
    for _ in range(npath):
        e = int(rng.integers(0, nsta))
        s = int(rng.integers(0, nsta))
        if s == e:
            s = (s + 1) % nsta
        rows.append(dict(
            tt=float(rng.uniform(10, 100)),
            staname=names[s] + (" " if rng.random() < 0.2 else ""),   # trailing blanks
            stla=22.0 + s * 0.3 + (0.01 if rng.random() < 0.1 else 0.0),  # first one wins
            stlo=100.0 + s * 0.2,
            evtname=names[e] if e < nsta - 1 else "EVONLY",                # not a station
            evla=21.0 + e * 0.1, evlo=101.0 - e * 0.1,
            period=per[int(rng.integers(0, nper))],
            weight=float(rng.uniform(0.5, 1.0))))
    return rows


def _oracle_rows(oracle, rows):
    return oracle.srcrec_worklist([r["evtname"] for r in rows], [r["staname"] for r in rows],
                                  [r["stla"] for r in rows], [r["stlo"] for r in rows],
                                  [r["evla"] for r in rows], [r["evlo"] for r in rows],
                                  [r["period"] for r in rows], [r["tt"] for r in rows],
                                  [r["weight"] for r in rows])


def assert_matches_py(o, p):
    assert list(o["periods"]) == p["periods"]
    assert [s.rstrip(" ") for s in o["sta_name"]] == p["sta"]
    assert list(o["sta_lo"]) == p["lo"] and list(o["sta_la"]) == p["la"]
    assert len(o["pidx"]) == len(p["solves"])
    for s, (ip, j, sx, sy, recs) in enumerate(p["solves"]):
        assert (o["pidx"][s], o["sta"][s], o["srcx"][s], o["srcy"][s]) == (ip, j, sx, sy)
        r0, nr = int(o["rec_off"][s]), int(o["nrec"][s])
        assert nr == len(recs)
        for q, (rx, ry, tt, w, m) in enumerate(recs):
            k = r0 + q
            assert (o["recx"][k], o["recy"][k], o["tt"][k], o["weight"][k], o["path"][k]) == \
                (rx, ry, tt, w, m)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_oracle_worklist_matches_restatement(oracle, seed):
    rows = tricky_rows(seed)
    o = _oracle_rows(oracle, rows)
    p = py_worklist(rows)
    assert_matches_py(o, p)
    # period 0 gets no solve (get_periods_by_src's zero-initialised list)
    assert 0.0 in p["periods"] and all(p["periods"][ip] != 0.0 for ip, *_ in p["solves"])


def _read_py(fname):
    with open(fname) as f:
        rows = list(csv.DictReader(f))
    conv = lambda r: dict(tt=float(r["tt"]), staname=r["staname"], stla=float(r["stla"]),
                          stlo=float(r["stlo"]), evtname=r["evtname"], evla=float(r["evla"]),
                          evlo=float(r["evlo"]), period=float(r["period"]),
                          weight=float(r.get("weight", 1.0)))
    return [conv(r) for r in rows]


def _csv_files():
    files = [os.path.join(GOLDEN, "config1_src_rec.csv")]
    for sub in ("00_checkerboard_iso/src_rec_file_ph.csv", "00_checkerboard_iso/src_rec_file_gr.csv",
                "03_checkerboard_2d/src_rec_file_ph.csv"):
        f = os.path.join(EXAMPLES, sub)
        if os.path.exists(f):
            files.append(f)
    return files


@pytest.mark.parametrize("fname", _csv_files(), ids=os.path.basename)
def test_native_csv_reader(sg, oracle, fname):
    """The native reader parses the reference's layout like Python's csv
    module, and its period and station tables are the oracle's."""
    rows = _read_py(fname)
    t = sg.SrcRec.read_csv(fname)
    p = t.paths()
    assert np.array_equal(p["tt"], [r["tt"] for r in rows])
    assert np.array_equal(p["period"], [r["period"] for r in rows])
    assert np.array_equal(p["weight"], [r["weight"] for r in rows])
    o = _oracle_rows(oracle, rows)
    assert np.array_equal(t.periods(), o["periods"])
    names, lo, la = t.stations()
    assert names == [s.rstrip(" ") for s in o["sta_name"]]
    assert np.array_equal(lo, o["sta_lo"]) and np.array_equal(la, o["sta_la"])
    t.close()


def test_csv_write_read_round_trip(sg, tmp_path):
    rows = tricky_rows(3)
    t = sg.SrcRec.from_arrays(*[[r[k] for r in rows] for k in
                                ("evtname", "staname", "stla", "stlo", "evla", "evlo", "period",
                                 "tt")], weight=[r["weight"] for r in rows])
    tt = np.array([r["tt"] for r in rows]) * 1.001
    fn = tmp_path / "iter.csv"
    t.write_csv(fn, tt)
    lines = open(fn).read().splitlines()
    assert lines[0] == "tt,staname,stla,stlo,evtname,evla,evlo,period,weight,dist,vel"
    back = sg.SrcRec.read_csv(fn)
    p = back.paths()
    assert np.allclose(p["tt"], tt, atol=5e-7) and np.allclose(p["period"], [r["period"] for r in rows])
    f = lines[1].split(",")
    assert len(f[2].split(".")[1]) == 4 and len(f[0].split(".")[1]) == 6   # F9.4, F0.6
    dist = float(f[9])
    lat0, lon0, lat1, lon1 = rows[0]["stla"], rows[0]["stlo"], rows[0]["evla"], rows[0]["evlo"]
    d2r = float(np.float32(3.14159265359)) / 180.0
    a = math.sin((lat0 - lat1) * d2r * 0.5) ** 2 + math.sin((lon1 - lon0) * d2r * 0.5) ** 2 * \
        math.cos(lat0 * d2r) * math.cos(lat1 * d2r)
    assert abs(dist - 6371.0 * 2 * math.atan2(math.sqrt(a), math.sqrt(1 - a))) < 1e-4
    t.close()
    back.close()


def test_csv_reader_rejects_bad_input(sg, tmp_path):
    bad = tmp_path / "bad.csv"
    bad.write_text("tt,staname,stla,stlo,evtname,evla,period\n1,A,1,2,B,3,4\n")   # no evlo
    with pytest.raises(sg.SurfattError):
        sg.SrcRec.read_csv(bad)
    bad.write_text("tt,staname,stla,stlo,evtname,evla,evlo,period\n1,A,1,2,B,3,x,4\n")
    with pytest.raises(sg.SurfattError):
        sg.SrcRec.read_csv(bad)
    with pytest.raises(sg.SurfattError):
        sg.SrcRec.read_csv(tmp_path / "missing.csv")
