"""The C-ABI library builds, loads and exports every entry point the header
declares (no GPU needed: nothing is called that touches a device)."""
import ctypes
import os
import re

from voxel_ma_gb300 import _lib

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^\s*(?:const\s+)?[\w\*]+\s+\*?\s*(vc_\w+)\s*\(", src, re.M))
    return names


def test_every_declared_symbol_is_exported():
    lib = _lib.load()
    declared = _declared()
    assert len(declared) >= 20
    for name in sorted(declared):
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, name


def test_status_strings_without_gpu():
    lib = _lib.load()
    assert lib.vc_version() >= 100
    for s in range(7):
        assert lib.vc_status_string(s)


def test_null_context_is_rejected_not_crashed():
    lib = _lib.load()
    assert lib.vc_ctx_sync(None) == _lib.VC_ERR_ARG
    assert lib.vc_ctx_create(None, 0) == _lib.VC_ERR_ARG
    out = ctypes.c_int64()
    assert lib.vc_extract_sites(None, ctypes.byref(out)) == _lib.VC_ERR_ARG
