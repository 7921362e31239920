"""The C-ABI library builds, loads without a GPU and exports every function
that include/surfatt_gb300.h declares (no compute calls here)."""
import ctypes
import os
import re

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "surfatt_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = set()
    for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*([a-z_][a-z0-9_]*)\s*\(",
                         src, flags=re.M):
        names.add(m.group(1))
    return names


def test_header_symbols_exported(sg):
    names = _declared()
    assert "fsm_uw_ps_lonlat_2d_" in names and "mask_" in names
    lib = ctypes.CDLL(sg.library_path())
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(sg.EXPORTED) <= names


def test_library_reports_no_device_without_gpu(sg):
    import torch
    if torch.cuda.is_available():
        return
    h = ctypes.c_void_p()
    st = sg.lib().surfatt_engine_create(ctypes.byref(h), 0, 0)
    assert st == sg.CUDA_ERROR


def test_smooth_rejects_bad_grids_before_the_device(sg):
    """gaussian_smooth_geo_2's argument checks run on the host, before any
    device call: grids the reference would read outside of or divide by zero
    on are SURFATT_BAD_ARG (no GPU needed)."""
    import numpy as np
    L = sg.lib()
    dp = ctypes.POINTER(ctypes.c_double)
    L.surfatt_gaussian_smooth_geo_2.argtypes = [dp, ctypes.c_int, ctypes.c_int, dp, dp,
                                                ctypes.c_double, dp]

    def call(lons, lats, sigma):
        lons, lats = np.asarray(lons, float), np.asarray(lats, float)
        d = np.zeros(len(lons) * len(lats))
        o = np.zeros_like(d)
        p = lambda a: a.ctypes.data_as(dp)
        return L.surfatt_gaussian_smooth_geo_2(p(d), len(lons), len(lats), p(lons), p(lats),
                                               sigma, p(o))

    x, y = 100 + 0.05 * np.arange(8), 30 + 0.05 * np.arange(6)
    assert call(x[::-1], y, 0.1) == sg.BAD_ARG          # decreasing longitudes
    assert call(x, y[::-1], 0.1) == sg.BAD_ARG          # decreasing latitudes
    xn = x.copy()
    xn[5] += 0.01
    assert call(xn, y, 0.1) == sg.BAD_ARG               # non-uniform spacing
    assert call(x, y, 0.0) == sg.BAD_ARG                # sigma = 0 (0/0 weights)
    assert call(x, y, float("nan")) == sg.BAD_ARG
    assert call(x[:1], y, 0.1) == sg.BAD_ARG            # one column: no dx
    assert call(x, 85 + 1.0 * np.arange(6), 0.1) == sg.BAD_ARG  # reaches the pole


def test_projection_locate_failure_before_the_device(sg):
    """inv_grid_iso_ with a model node outside the inversion grids: with the
    `stop` switch off the status is SURFATT_BAD_ARG, decided on the host
    before any device call (no GPU needed)."""
    import numpy as np
    sg.set_exit_on_boundary(False)
    try:
        vx, vy, vz = np.arange(7.0), np.arange(6.0), np.arange(5.0)
        xinv = np.asfortranarray(np.array([[1.5, 2.0, 3.0, 7.5]]).T)
        yinv = np.asfortranarray(np.array([[-1.5, 2.0, 4.0, 6.5]]).T)
        zinv = np.asfortranarray(np.array([[-1.0, 1.0, 3.0, 5.0]]).T)
        try:
            sg.inv_grid_iso(xinv, yinv, zinv, np.zeros((7, 6, 5)), vx, vy, vz)
            raise AssertionError("expected SurfattError")
        except sg.SurfattError as e:
            assert e.status == sg.BAD_ARG
    finally:
        sg.set_exit_on_boundary(True)


def test_projection_locate_failure_stops_like_the_reference(sg):
    """With the switch on (default) the drop-in prints the reference's
    message with the node and ends the process with status 0 (`stop`)."""
    import subprocess
    import sys
    code = (
        "import sys, numpy as np; sys.path.insert(0, %r); import surfatt_gb300 as sg\n"
        "vx, vy, vz = np.arange(7.0), np.arange(6.0), np.arange(5.0)\n"
        "xi = np.asfortranarray(np.array([[1.5, 2.0, 3.0, 7.5]]).T)\n"
        "yi = np.asfortranarray(np.array([[-1.5, 2.0, 4.0, 6.5]]).T)\n"
        "zi = np.asfortranarray(np.array([[-1.0, 1.0, 3.0, 5.0]]).T)\n"
        "sg.inv_grid_iso(xi, yi, zi, np.zeros((7, 6, 5)), vx, vy, vz)\n"
        "print('not reached')\n") % os.path.join(ROOT, "surfatt-iso_gb300")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert "I cannot locate the receiver in the domain." in r.stdout
    assert "not reached" not in r.stdout
    vals = [float(v) for v in r.stdout.split("domain.")[1].split()]
    assert vals == [1.0, 1.0, 1.0]


# C layout of the ISO_C_BINDING kinds the Fortran module uses (LP64)
_F_KINDS = {"integer(c_int)": (4, 4), "type(c_ptr)": (8, 8), "real(c_double)": (8, 8),
            "integer(c_size_t)": (8, 8), "integer(c_long_long)": (8, 8)}


def _fortran_types():
    """{type name: [(kind, field), ...]} of the bind(c) derived types of
    include/surfatt_gpu.f90, in declaration order."""
    src = open(os.path.join(ROOT, "include", "surfatt_gpu.f90")).read()
    out = {}
    for m in re.finditer(r"type\s*,\s*bind\(c\)\s*::\s*(\w+)(.*?)end\s+type", src, flags=re.S | re.I):
        fields = []
        for line in m.group(2).splitlines():
            line = line.split("!")[0].strip()
            if not line:
                continue
            kind, _, names = line.partition("::")
            for name in names.split(","):
                fields.append((kind.strip().lower().replace(" ", ""), name.strip()))
        out[m.group(1)] = fields
    return out


def test_fortran_binding_matches_c_structs(tmp_path):
    """The module's derived types have the C structs' fields in the same
    order with the same sizes and offsets (what bind(c) relies on): a C
    probe prints offsetof / sizeof of every field the module names, which
    must equal the offsets the module's kinds give under C layout rules."""
    import subprocess
    types = _fortran_types()
    assert set(types) == {"surfatt_problem_t", "surfatt_result_t"}
    probe = ['#include <stdio.h>', '#include <stddef.h>', '#include "surfatt_gb300.h"',
             "int main(void) {"]
    expect = []
    for t, fields in types.items():
        off = 0
        for kind, name in fields:
            size, align = _F_KINDS[kind]
            off = (off + align - 1) // align * align
            expect.append(f"{t}.{name} {off} {size}")
            probe.append(f'  printf("{t}.{name} %zu %zu\\n", offsetof({t}, {name}), '
                         f'sizeof((({t}*)0)->{name}));')
            off += size
        total = (off + 7) // 8 * 8
        expect.append(f"{t} {total}")
        probe.append(f'  printf("{t} %zu\\n", sizeof({t}));')
    probe.append("  return 0;\n}\n")
    c = tmp_path / "probe.c"
    c.write_text("\n".join(probe))
    exe = tmp_path / "probe"
    subprocess.check_call(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(c), "-o",
                           str(exe)])
    got = subprocess.check_output([str(exe)], text=True).split("\n")
    assert [g for g in got if g] == expect


def test_fortran_binding_names_exported_symbols():
    """Every bind(c, name=...) of the module is a function the header declares."""
    src = open(os.path.join(ROOT, "include", "surfatt_gpu.f90")).read()
    names = set(re.findall(r'bind\(c,\s*name="(\w+)"\)', src))
    assert names and names <= _declared()
