"""The C-ABI library builds, loads and exports every symbol include/gbmhd.h declares (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "gbmhd.h")).read()
    return sorted(set(re.findall(r"\b(gbmhd_[a-z_]+)\s*\(", txt)))


def test_header_and_binding_agree():
    from gbmhd import lib
    assert set(declared_symbols()) == set(lib.SYMBOLS)


def test_library_exports_all_symbols(gpu_lib):
    for s in declared_symbols():
        assert hasattr(gpu_lib, s), s
    assert gpu_lib.gbmhd_version() == 1


def test_create_rejects_bad_input_without_gpu_work(gpu_lib):
    from gbmhd.lib import DofMap, Mesh, Params
    h = ctypes.c_void_p()
    rc = gpu_lib.gbmhd_create(ctypes.byref(h), None, None, None)
    assert rc < 0
    assert b"NULL" in gpu_lib.gbmhd_last_error(None)
    m = Mesh(0, None)
    rc = gpu_lib.gbmhd_create(ctypes.byref(h), ctypes.byref(m), ctypes.byref(DofMap()), ctypes.byref(Params()))
    assert rc < 0 and b"no cells" in gpu_lib.gbmhd_last_error(None)
