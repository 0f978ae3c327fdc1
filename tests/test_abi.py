"""The C-ABI library: it loads, exports exactly what include/beastgb.h declares, and fails
cleanly (no crash, a status code and a message) when no GPU is present or inputs are bad.
These tests make no compute call."""
import ctypes as C
import os
import re
import subprocess

import pytest

from beastgpu_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "beastgb.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(bgb_[a-z_0-9]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from beastgpu_gb300.csrc import build
        build.build()
    return _lib.load()


def test_header_declares_the_expected_entry_points():
    names = declared_functions()
    for must in ("bgb_create", "bgb_destroy", "bgb_assemble", "bgb_assemble_batch", "bgb_classify_block",
                 "bgb_local_matrices", "bgb_last_error", "bgb_assemble_curve", "bgb_local_matrices_curve"):
        assert must in names


def test_every_declared_symbol_is_exported(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"


def test_no_undeclared_exports(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = sorted(set(re.findall(r"\b[TW] (bgb_[a-z_0-9]+)$", out, flags=re.M)))
    assert exported == declared_functions()


def test_abi_version(lib):
    assert lib.bgb_abi_version() == _lib.ABI_VERSION == 3
    n = lib.bgb_tile_info(None, 0)
    assert n >= 4


def test_invalid_handle_is_an_error_not_a_crash(lib):
    rc = lib.bgb_assemble(None, None, None, None, None, 0, None, 0, 1, 0, -1, None, None)
    assert rc == -1
    assert b"handle" in lib.bgb_last_error()
    rc = lib.bgb_assemble_curve(None, None, None, None, None, 0, None, 0, 1, 0, -1, None, None)
    assert rc == -1
    assert lib.bgb_destroy(None) == 0
    assert lib.bgb_abort(None) == -1


def test_create_without_gpu_reports_cuda_error(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    rc = lib.bgb_create(C.byref(h), None)
    assert rc == -3 and not h
    assert len(lib.bgb_last_error()) > 0
