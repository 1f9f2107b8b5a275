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
