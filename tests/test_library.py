"""The C-ABI library builds, loads without a GPU and exports every declared symbol."""

import ctypes
import os
import re

import pytest

from regridding_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "regrid_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return ctypes.CDLL(_build.LIB)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "rg_apply" in syms and "rg_build_conservative_2d" in syms
    assert len(syms) >= 15


def test_every_declared_symbol_is_exported(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_binding_covers_header():
    assert set(_lib.SIGNATURES) == set(declared_symbols())


def test_version_and_error_buffer(lib):
    assert lib.rg_version() >= 100
    buf = ctypes.create_string_buffer(64)
    n = lib.rg_last_error(buf, 64)
    assert n >= 0 and len(buf.value) <= 63


def test_argument_errors_need_no_gpu():
    """Argument validation happens before any CUDA call."""
    lib = _lib.load()
    st = lib.rg_cell_area_2d(None, None, 1, 5, None, None)
    assert st == _lib.RG_ERR_ARG
    assert "2x2" in _lib.last_error()
    st = lib.rg_locate_2d(None, None, 4, 4, None, None, 1, 7, None, None, None)
    assert st == _lib.RG_ERR_ARG
    st = lib.rg_apply(None, None, 0, None, 0, 1, 0, None)
    assert st == _lib.RG_ERR_ARG


def test_product_refuses_without_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np

    import regridding_gb300 as rg

    with pytest.raises(rg.RegridError):
        rg.find_indices((np.linspace(0, 1, 5),), (np.linspace(0, 1, 3),))


def test_batch_and_option_arguments_need_no_gpu():
    L = _lib.load()
    for name, args in _lib.SIGNATURES.items():
        getattr(L, name).argtypes = args
    out = (ctypes.c_void_p * 1)()
    status = (ctypes.c_int * 1)()
    assert L.rg_build_conservative_2d_batch(0, None, None, None, None, None, None, None, None, None, None, out,
                                            status) == _lib.RG_ERR_ARG
    assert L.rg_build_conservative_2d_batch(1, None, None, None, None, None, None, None, None, None, None, out,
                                            status) == _lib.RG_ERR_ARG
    assert L.rg_set_sweep_chunk(-1) == _lib.RG_ERR_ARG
    assert L.rg_set_sweep_chunk(32) == _lib.RG_OK
    assert L.rg_weights_check(None, None) == _lib.RG_ERR_ARG
    assert L.rg_weights_set_input_shape(None, 1, 1) == _lib.RG_ERR_ARG
    assert L.rg_weights_device_bytes(None, None) == _lib.RG_ERR_ARG
    assert L.rg_conservative_2d_grad_output(None, None, None, 2, 2, None, None, 2, 2, None, None, None, 0, 1,
                                            None, None, None, None) == _lib.RG_ERR_ARG


def test_hash64_is_a_host_function():
    """rg_hash64 runs on the host (no GPU): deterministic, seed- and
    content-sensitive, and the same on both sides of the 4 MiB segmented
    path's threshold whatever thread count hashes the segments."""
    import numpy as np

    L = _lib.load()

    def h(a, seed=7):
        out = ctypes.c_uint64()
        assert L.rg_hash64(ctypes.c_void_p(a.ctypes.data), a.nbytes, seed, ctypes.byref(out)) == _lib.RG_OK
        return out.value

    rng = np.random.default_rng(0)
    for n in (0, 1, 31, 32, 33, 1000, (4 << 20) // 8, (4 << 20) // 8 + 1, 3_000_000):
        a = rng.random(n)
        assert h(a) == h(a.copy())
        if n:
            b = a.copy()
            b[n // 2] = np.nextafter(b[n // 2], 2.0)
            assert h(b) != h(a)
            assert h(a, 8) != h(a, 7)
    out = ctypes.c_uint64()
    assert L.rg_hash64(None, 8, 0, ctypes.byref(out)) == _lib.RG_ERR_ARG
    assert L.rg_hash64(None, 0, 0, ctypes.byref(out)) == _lib.RG_OK


def test_hash64x2_equals_two_hash64():
    """rg_hash64x2 gives rg_hash64's two values in one pass, below and above
    the segmented path's 4 MiB threshold (the serving cache keys use it)."""
    import numpy as np

    L = _lib.load()
    rng = np.random.default_rng(1)
    for n in (0, 5, 32, 999, 4 << 20, (4 << 20) + 3, 9_000_001):
        a = rng.integers(0, 256, n, dtype=np.uint8)
        pair = (ctypes.c_uint64 * 2)()
        assert L.rg_hash64x2(ctypes.c_void_p(a.ctypes.data), n, 11, 13, pair) == _lib.RG_OK
        for seed, got in ((11, pair[0]), (13, pair[1])):
            one = ctypes.c_uint64()
            assert L.rg_hash64(ctypes.c_void_p(a.ctypes.data), n, seed, ctypes.byref(one)) == _lib.RG_OK
            assert got == one.value


def test_debug_library_builds_with_every_symbol():
    """The RG_DEBUG variant (bounds-checked grid reads in the builds) compiles
    and exports every entry point the header declares."""
    import ctypes

    from regridding_gb300 import _build

    path = _build.build(debug=True)
    assert path == _build.LIB_DEBUG
    dbg = ctypes.CDLL(path)
    for name in declared_symbols():
        assert hasattr(dbg, name), name
    assert dbg.rg_version() == _lib.load().rg_version()
