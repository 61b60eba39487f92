"""The C-ABI library loads and exports every symbol include/fdtd_gb300.h
declares, and the ctypes mirrors have the C struct sizes.  No compute calls
(this runs without a GPU)."""

import ctypes
import os
import re

import pytest
import torch

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


def test_compact_material_arguments_without_gpu(lib):
    """The compact material fields are validated before any CUDA call: at most
    256 table rows, a table for any count, an index unless the table has one
    row; an unaligned index or nz not a multiple of 16 is not an error (the
    plan reads the full arrays)."""
    if torch.cuda.is_available():
        pytest.skip("checks the CPU-only path")
    fake = 1 << 20  # never dereferenced: validation fails or the first CUDA call does

    def desc(**kw):
        d = _native.GridDesc()
        d.abi_version = _native.ABI_VERSION
        d.precision = _native.FLOAT32
        d.nx = d.ny = d.nz = 16
        d.courant = 0.5
        d.E = d.H = d.inv_eps = d.inv_mu = fake
        for k, v in kw.items():
            setattr(d, k, v)
        return d

    plan = ctypes.c_void_p()
    create = lambda d: lib.fdtd_plan_create(ctypes.byref(d), ctypes.byref(plan))  # noqa: E731
    assert create(desc(n_eps_table=257, eps_table=fake, eps_index=fake)) == 1
    assert create(desc(n_eps_table=-1)) == 1
    assert create(desc(n_eps_table=2, eps_table=fake)) == 1  # no index for two rows
    assert create(desc(n_mu_table=1)) == 1  # no table
    assert create(desc(materials_scaled=1)) == 2  # float64 plans only
    # valid compact fields pass validation; the CPU-only host then fails at the first CUDA call
    assert create(desc(n_eps_table=3, eps_table=fake, eps_index=fake, n_mu_table=1, mu_table=fake)) == 3
