"""The C-ABI library builds for sm_103a, loads, and exports every symbol include/*.h declares (CPU only)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(vh_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__

    __graft_entry__.build()
    from voxhenry_gb300 import _lib

    return _lib.load()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "vh_matvec" in names and "vh_geom_create" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(lib):
    from voxhenry_gb300 import _lib

    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_no_device_is_reported_without_gpu(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert lib.vh_ctx_create(0, ctypes.byref(h)) == 7       # VH_ERR_NO_DEVICE, no crash
    assert lib.vh_status_string(3) == b"unsupported"
