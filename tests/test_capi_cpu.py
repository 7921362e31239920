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
