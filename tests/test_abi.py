"""The C-ABI library loads and exports every symbol include/fdtd_gb300.h
declares, and the ctypes mirrors have the C struct sizes.  No compute calls
(this runs without a GPU)."""

import ctypes
import os
import re

import pytest

from fdtd_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fdtd_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fdtd_[A-Za-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_native.LIB_PATH):
        from fdtd_gb300 import build

        build.build()
    return _native.load()


def test_header_declares_expected_entry_points():
    names = declared_functions()
    for n in ("fdtd_plan_create", "fdtd_plan_destroy", "fdtd_run", "fdtd_curl_E", "fdtd_curl_H"):
        assert n in names


def test_every_declared_symbol_is_exported(lib):
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared in the header but not exported"
        assert name in _native.SIGNATURES, f"{name} has no ctypes signature"


def test_struct_sizes_match(lib):
    for i, s in enumerate([_native.GridDesc, _native.BoundaryDesc, _native.ItemDesc, _native.DftDesc,
                           _native.RunArgs, _native.CaptureArgs, _native.AdjointArgs]):
        assert lib.fdtd_abi_sizeof(i) == ctypes.sizeof(s), s.__name__


def test_status_strings(lib):
    assert lib.fdtd_status_string(0) == b"ok"
    assert lib.fdtd_status_string(5) == b"out of range"
    assert lib.fdtd_status_string(99) == b"unknown status"


def test_argument_errors_without_gpu(lib):
    """Validation runs before any CUDA call, so it works on a CPU-only host."""
    d = _native.GridDesc()
    d.abi_version = 999
    plan = ctypes.c_void_p()
    assert lib.fdtd_plan_create(ctypes.byref(d), ctypes.byref(plan)) == 1
    d.abi_version = _native.ABI_VERSION
    d.nx = d.ny = d.nz = 4
    assert lib.fdtd_plan_create(ctypes.byref(d), ctypes.byref(plan)) == 1  # null field pointers
    assert lib.fdtd_run(None, None, None) == 1
    assert lib.fdtd_curl_E(0, None, None, 1, 1, 1, None) == 1
    assert lib.fdtd_field_stats(None, None, None, None) == 1
