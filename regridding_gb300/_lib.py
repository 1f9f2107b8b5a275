"""ctypes binding of ``libregrid_gb300.so`` (declared in ``include/regrid_gb300.h``).

The library is the only compute path: if it cannot be loaded, or no CUDA
device is present, every call raises instead of falling back to the CPU.
"""

from __future__ import annotations

import ctypes
import os
import threading

from . import _build

RG_OK = 0
RG_ERR_ARG = 1
RG_ERR_CUDA = 2
RG_ERR_ALLOC = 3
RG_ERR_WALK = 4
RG_ERR_UNSUPPORTED = 5

RG_F32 = 0
RG_F64 = 1
RG_FILL_GUESS_MEDIAN = 0
RG_FILL_GUESS_SLICE = 1
RG_FILL_GUESS_FULL = 2
RG_ACC_EXACT = 0
RG_ACC_FAST = 1
RG_ACC_COMPENSATED = 2
RG_ACC = {"exact": RG_ACC_EXACT, "fast": RG_ACC_FAST, "compensated": RG_ACC_COMPENSATED}
RG_BOUNDS = {"extrapolate": 0, "nan": 1, "raise": 2}

_P = ctypes.c_void_p
_I = ctypes.c_int64
_C = ctypes.c_int

# name -> argument types (all return int status unless listed in _RESTYPE)
SIGNATURES = {
    "rg_version": [],
    "rg_last_error": [ctypes.c_char_p, ctypes.c_size_t],
    "rg_build_conservative_2d": [_P, _P, _I, _I, _P, _P, _I, _I, _P, _P, ctypes.POINTER(_P)],
    "rg_set_sweep_chunk": [_I],
    "rg_interp_linear": [_P, _I, _I, _I, _P, _P, _I, _I, _I, _P, _P],
    "rg_device_attributes": [_P, _C],
    "rg_copy_from_host": [_P, _P, _I, _P],
    "rg_hash64x2": [_P, _I, ctypes.c_uint64, ctypes.c_uint64, _P],
    "rg_fill_gauss_seidel": [_P, _C, _P, _I, _I, _I, _P, _C, _I, _P],
    "rg_fill_median": [_P, _C, _P, _I, _I, _P, _P],
    "rg_build_conservative_2d_batch": [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "rg_weights_from_coo": [_P, _P, _P, _I, _I, _I, _P, ctypes.POINTER(_P)],
    "rg_weights_info": [_P, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)],
    "rg_weights_set_output_shape": [_P, _I, _I],
    "rg_weights_export_coo": [_P, _P, _P, _P, _P],
    "rg_weights_free": [_P, _P],
    "rg_weights_set_input_shape": [_P, _I, _I],
    "rg_weights_check": [_P, _P],
    "rg_apply": [_P, _P, _C, _P, _C, _I, _C, _P],
    "rg_apply_transpose": [_P, _P, _C, _P, _C, _I, _C, _P],
    "rg_apply_host": [_P, _P, _C, _P, _C, _I, _C, _I, _P],
    "rg_cell_area_2d": [_P, _P, _I, _I, _P, _P],
    "rg_cell_length_1d": [_P, _I, _I, _P, _P],
    "rg_locate_2d": [_P, _P, _I, _I, _P, _P, _I, _C, _P, _P, _P],
    "rg_locate_2d_noalloc": [_P, _P, _I, _I, _P, _P, _I, _P, _P, _P],
    "rg_find_indices_1d": [_P, _I, _I, _P, _I, _I, _I, _C, _I, _P, _P],
    "rg_multilinear_1d": [_P, _I, _I, _P, _P, _I, _I, _I, _P, _I, _C, _P, _P, _P, ctypes.POINTER(_I), _P],
    "rg_conservative_1d": [_P, _I, _I, _P, _I, _I, _I, _P, _I, _I, _P, _P, _P, _P, _P],
    "rg_transpose_conservative_scale": [_P, _P, _P, _I, _P, _I, _P, _I, _P, _P, _P],
    "rg_weights_device_bytes": [_P, ctypes.POINTER(_I)],
    "rg_conservative_2d_grad_output": [_P, _P, _P, _I, _I, _P, _P, _I, _I, _P, _P, _P, _C, _I, _P, _P, _P, _P],
    "rg_hash64": [_P, _I, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)],
}

_lock = threading.Lock()
_lib = None


class RegridError(RuntimeError):
    """A failure reported by the CUDA library."""


def debug_requested() -> bool:
    """RG_DEBUG=1 selects the bounds-checked debug library."""
    return os.environ.get("RG_DEBUG", "") not in ("", "0")


def library_path() -> str:
    return _build.LIB_DEBUG if debug_requested() else _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the CUDA library: the release build,
    or with RG_DEBUG=1 the bounds-checked debug build."""
    global _lib
    with _lock:
        if _lib is None:
            debug = debug_requested()
            path = library_path()
            if not os.path.exists(path):
                if not build_if_missing:
                    raise RegridError(f"{path} is missing; run regridding_gb300._build.build(debug={debug})")
                _build.build(debug=debug)
            lib = ctypes.CDLL(path)
            for name, args in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.argtypes = args
                fn.restype = ctypes.c_int
            _lib = lib
    return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    load().rg_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int, what: str) -> None:
    if status == RG_OK:
        return
    msg = last_error()
    if status == RG_ERR_ARG:
        raise ValueError(f"{what}: {msg}")
    raise RegridError(f"{what} failed (status {status}): {msg}")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)
