"""ctypes binding of ``libfdtd_gb300.so`` (the C ABI declared in include/fdtd_gb300.h).

The library is loaded lazily on first use.  There is no fallback: if the
shared library is missing or cannot be loaded, every compute entry point
raises ``RuntimeError`` naming the cause.
"""

import ctypes
import os

LIB_NAME = "libfdtd_gb300.so"
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), LIB_NAME)

ABI_VERSION = 5
MAX_BOUNDARIES = 9

FLOAT32, FLOAT32C, FLOAT64 = 0, 1, 2
BOUNDARY_PML, BOUNDARY_PERIODIC = 0, 1
ITEM_OBJECT, ITEM_ABSORBING, ITEM_ANISOTROPIC, ITEM_SOFT, ITEM_HARD, ITEM_FEEDBACK = 0, 1, 2, 3, 4, 5
STATS_STATIC_MAX_ROWS = 1024  # FDTD_STATS_STATIC_MAX_ROWS

STATUS = {
    0: "ok",
    1: "invalid argument",
    2: "unsupported configuration",
    3: "CUDA error",
    4: "non-finite field value",
    5: "out of range",
}

c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_void_p = ctypes.c_void_p


class BoundaryDesc(ctypes.Structure):
    _fields_ = [
        ("kind", c_int32), ("axis", c_int32), ("high", c_int32), ("thickness", c_int32),
        ("psi_E", c_void_p), ("psi_H", c_void_p),
        ("b_E", c_void_p), ("c_E", c_void_p), ("b_H", c_void_p), ("c_H", c_void_p),
    ]


class ItemDesc(ctypes.Structure):
    _fields_ = [
        ("kind", c_int32), ("comp", c_int32), ("column", c_int32), ("source", c_int32),
        ("lo", c_int32 * 3), ("hi", c_int32 * 3),
        ("weight", ctypes.c_double),
        ("coef", c_void_p * 3),
        ("aux", c_int32), ("reserved", c_int32),
    ]


class DftDesc(ctypes.Structure):
    _fields_ = [
        ("lo", c_int32 * 3), ("hi", c_int32 * 3),
        ("n_freq", c_int32), ("phase_offset", c_int32),
        ("acc", c_void_p),
    ]


class GridDesc(ctypes.Structure):
    _fields_ = [
        ("abi_version", c_int32), ("precision", c_int32),
        ("nx", c_int32), ("ny", c_int32), ("nz", c_int32), ("x_chunk", c_int32),
        ("variant", c_int32), ("tile_rows", c_int32), ("stages", c_int32), ("pml_mode", c_int32),
        ("courant", ctypes.c_double),
        ("E", c_void_p), ("H", c_void_p), ("E_lo", c_void_p), ("H_lo", c_void_p),
        ("inv_eps", c_void_p), ("inv_mu", c_void_p),
        ("n_boundaries", c_int32),
        ("boundaries", BoundaryDesc * MAX_BOUNDARIES),
        ("n_objects", c_int32), ("objects", ctypes.POINTER(ItemDesc)),
        ("n_sources_E", c_int32), ("sources_E", ctypes.POINTER(ItemDesc)),
        ("n_sources_H", c_int32), ("sources_H", ctypes.POINTER(ItemDesc)),
        ("n_columns", c_int32),
        ("n_probe_cells", c_int32), ("probe_cells", c_void_p),
        ("n_dft", c_int32), ("dft", ctypes.POINTER(DftDesc)),
        ("n_phase_columns", c_int32),
        ("n_current_cells", c_int32), ("current_cells", c_void_p),
        ("grid_spacing", ctypes.c_double), ("materials_scaled", c_int32),
        ("eps_table", c_void_p), ("n_eps_table", c_int32), ("eps_index", c_void_p),
        ("mu_table", c_void_p), ("n_mu_table", c_int32), ("mu_index", c_void_p),
        ("step_fusion", c_int32), ("persistent", c_int32),
        ("E_alt", c_void_p), ("H_alt", c_void_p),
        ("psi_alt", (c_void_p * 2) * MAX_BOUNDARIES),
    ]


class RunArgs(ctypes.Structure):
    _fields_ = [
        ("n_steps", c_int64), ("half", c_int32), ("reserved", c_int32),
        ("wave", c_void_p), ("phase", c_void_p),
        ("trace_E", c_void_p), ("trace_H", c_void_p),
        ("trace_capacity", c_int64), ("record_E", c_int64), ("record_H", c_int64),
        ("trace_I", c_void_p), ("record_I", c_int64), ("step0", c_int64),
    ]


class CaptureArgs(ctypes.Structure):
    _fields_ = [
        ("detectors", c_int32), ("n_curl", c_int32),
        ("curl", ctypes.POINTER(c_void_p)),
    ]


class AdjointArgs(ctypes.Structure):
    _fields_ = [
        ("n_steps", c_int64), ("parity", c_int32), ("n_objects", c_int32),
        ("lam_E", c_void_p), ("lam_H", c_void_p),
        ("aux_E", (c_void_p * 2) * MAX_BOUNDARIES), ("aux_H", (c_void_p * 2) * MAX_BOUNDARIES),
        ("seed_E", c_void_p), ("seed_H", c_void_p), ("seed_row", c_int64),
        ("dft_grad", ctypes.POINTER(c_void_p)), ("phase", c_void_p),
        ("curl", ctypes.POINTER(c_void_p)), ("curl_row", c_int64),
        ("grad", ctypes.POINTER(c_void_p)),
    ]


# every symbol declared in include/fdtd_gb300.h with (restype, argtypes)
SIGNATURES = {
    "fdtd_plan_create": (c_int32, [ctypes.POINTER(GridDesc), ctypes.POINTER(c_void_p)]),
    "fdtd_plan_destroy": (c_int32, [c_void_p]),
    "fdtd_plan_status": (c_int32, [c_void_p, ctypes.POINTER(c_int32), c_int32, c_void_p]),
    "fdtd_selftest_bounded_wait": (c_int32, [ctypes.c_uint32, ctypes.POINTER(c_int32), c_void_p]),
    "fdtd_run": (c_int32, [c_void_p, ctypes.POINTER(RunArgs), c_void_p]),
    "fdtd_run_capture": (c_int32, [c_void_p, ctypes.POINTER(RunArgs), ctypes.POINTER(CaptureArgs), c_void_p]),
    "fdtd_adjoint_run": (c_int32, [c_void_p, ctypes.POINTER(AdjointArgs), c_void_p]),
    "fdtd_curl_E": (c_int32, [c_int32, c_void_p, c_void_p, c_int32, c_int32, c_int32, c_void_p]),
    "fdtd_curl_H": (c_int32, [c_int32, c_void_p, c_void_p, c_int32, c_int32, c_int32, c_void_p]),
    "fdtd_stats_scratch_bytes": (ctypes.c_size_t, [c_void_p]),
    "fdtd_field_stats": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "fdtd_field_stats_noalloc": (c_int32, [c_void_p, c_void_p, c_int32, c_void_p]),
    "fdtd_plan_tiling": (c_int32, [c_void_p, ctypes.POINTER(c_int64)]),
    "fdtd_plan_step_fusion": (c_int32, [c_void_p, ctypes.POINTER(c_int32), ctypes.POINTER(c_int32),
                                        ctypes.POINTER(c_int32)]),
    "fdtd_status_string": (ctypes.c_char_p, [c_int32]),
    "fdtd_last_cuda_error": (c_int32, []),
    "fdtd_abi_sizeof": (ctypes.c_size_t, [c_int32]),
}

_lib = None
_load_error = None


def load():
    """Return the loaded library; raise RuntimeError when it is unavailable."""
    global _lib, _load_error
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_NAME} is not built (expected at {LIB_PATH}); run "
            "`python -c 'import __graft_entry__ as g; g.build()'` or "
            "`python -m fdtd_gb300.build`.  The gb300 backend has no CPU fallback.")
    try:
        lib = ctypes.CDLL(LIB_PATH)
    except OSError as exc:  # pragma: no cover - depends on the machine
        _load_error = exc
        raise RuntimeError(f"cannot load {LIB_PATH}: {exc}") from exc
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc, what):
    """Raise RuntimeError for a non-zero fdtd_status."""
    if rc != 0:
        lib = load()
        msg = lib.fdtd_status_string(rc).decode()
        extra = ""
        if rc == 3:
            extra = f" (cudaError {lib.fdtd_last_cuda_error()})"
        raise RuntimeError(f"{what} failed: {msg}{extra}")


def ptr(t):
    """Device (or host) address of a tensor's first element, or None."""
    return None if t is None else t.data_ptr()
