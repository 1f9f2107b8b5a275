"""ORACLE — test infrastructure only.

CPU restatement of the upstream ``regridding`` loops (sun-data/regridding),
used by ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` to check and to time against.  The product package never imports
this module.

The compiled part (``regrid_oracle.c``) restates the Numba loops in C with
pure-Python (JIT-disabled) arithmetic order; this module binds it with ctypes
and restates the numpy-level steps (``_coalesce``) on top.  The golden
fixtures in ``tests/golden`` (made by running the upstream package itself)
pin both halves bit for bit.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libregrid_oracle.so")
_lock = threading.Lock()
_lib = None

MAXSIZE = np.iinfo(np.int64).max
"""``sys.maxsize``: the out-of-grid sentinel of the upstream 2D point locators."""


def build(force: bool = False) -> str:
    """Compile the C restatement with the recipe in ``oracle/Makefile``."""
    src = os.path.join(_HERE, "regrid_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "--no-print-directory"],
                       check=True)
    return _LIB_PATH


class _Triples(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("inp", ctypes.POINTER(ctypes.c_int64)),
        ("out", ctypes.POINTER(ctypes.c_int64)),
        ("val", ctypes.POINTER(ctypes.c_double)),
    ]


class _Grid(ctypes.Structure):
    _fields_ = [
        ("x", ctypes.POINTER(ctypes.c_double)),
        ("y", ctypes.POINTER(ctypes.c_double)),
        ("nx", ctypes.c_int64),
        ("ny", ctypes.c_int64),
    ]


def _load():
    global _lib
    with _lock:
        if _lib is None:
            build()
            lib = ctypes.CDLL(_LIB_PATH)
            P = ctypes.c_void_p
            I = ctypes.c_int64
            lib.orc_cell_area_2d.argtypes = [I, I, P, P, P]
            lib.orc_sweep_2d.argtypes = [I, I, P, P, I, I, P, P, P, ctypes.c_int,
                                         ctypes.POINTER(_Triples)]
            lib.orc_sweep_2d.restype = ctypes.c_int
            lib.orc_free.argtypes = [P]
            lib.orc_locate_many.argtypes = [I, I, P, P, I, P, P, ctypes.c_int, P, P]
            lib.orc_apply_f64.argtypes = [I, I, I, I, P, P, P, P, P]
            lib.orc_apply_f32in.argtypes = [I, I, I, I, P, P, P, P, P]
            lib.orc_apply_f32in_f32out.argtypes = [I, I, I, I, P, P, P, P, P]
            for name in ("orc_find_indices_searchsorted", "orc_find_indices_brute"):
                getattr(lib, name).argtypes = [I, I, P, I, I, P, I, I, P]
            lib.orc_multilinear_1d.argtypes = [I, I, P, I, I, P, I, P, P, I, P, P, P, P]
            lib.orc_conservative_1d.argtypes = [I, P, I, P, P, I, P, P, P, P]
            lib.orc_conservative_1d.restype = I
            lib.orc_fill_gauss_seidel_f64.argtypes = [I, I, I, P, P, I]
            lib.orc_fill_gauss_seidel_f32.argtypes = [I, I, I, P, P, I]
            _lib = lib
    return _lib


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


# --------------------------------------------------------------------------
# 2D conservative
# --------------------------------------------------------------------------


def cell_area_2d(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """``grid_volume`` (regridding/_weights/_weights_conservative_2d/_grids.py:50-140)."""
    x, y = _f64(x), _f64(y)
    nx, ny = x.shape
    out = np.empty((nx - 1, ny - 1), dtype=np.float64)
    _load().orc_cell_area_2d(nx, ny, _ptr(x), _ptr(y), _ptr(out))
    return out


def sweep_2d(grid_input, grid_output, weights_input=None, nthreads: int = 0):
    """Raw (unmerged) triples of ``weights_conservative_2d`` in upstream emission order.

    Follows regridding/_weights/_weights_conservative_2d/_weights_conservative_2d.py:80-126
    up to (and including) ``_compact_rows`` (:27-73).
    """
    xi, yi = (_f64(a) for a in grid_input)
    xo, yo = (_f64(a) for a in grid_output)
    w = None if weights_input is None else _f64(np.broadcast_to(weights_input, (xi.shape[0] - 1, xi.shape[1] - 1)))
    res = _Triples()
    lib = _load()
    rc = lib.orc_sweep_2d(xi.shape[0], xi.shape[1], _ptr(xi), _ptr(yi),
                          xo.shape[0], xo.shape[1], _ptr(xo), _ptr(yo),
                          _ptr(w), int(nthreads), ctypes.byref(res))
    n = res.n
    try:
        if rc != 0:
            raise RuntimeError(f"oracle sweep failed with status {rc}")
        ind_in = np.ctypeslib.as_array(res.inp, shape=(max(n, 1),))[:n].copy()
        ind_out = np.ctypeslib.as_array(res.out, shape=(max(n, 1),))[:n].copy()
        val = np.ctypeslib.as_array(res.val, shape=(max(n, 1),))[:n].copy()
    finally:
        for p in (res.inp, res.out, res.val):
            if p:
                lib.orc_free(ctypes.cast(p, ctypes.c_void_p))
    return ind_in, ind_out, val


def coalesce(indices_input, indices_output, values):
    """``_coalesce`` (regridding/_weights/_weights_arrays.py:44-73), restated in numpy."""
    if values.shape[0] == 0:
        return indices_input, indices_output, values
    base_input = np.int64(indices_input.min())
    base_output = np.int64(indices_output.min())
    span_output = np.int64(indices_output.max()) - base_output + 1
    key = (indices_input - base_input) * span_output + (indices_output - base_output)
    order = np.argsort(key, kind="stable")
    key = key[order]
    values = values[order]
    boundary = np.empty(key.shape[0], dtype=bool)
    boundary[0] = True
    np.not_equal(key[1:], key[:-1], out=boundary[1:])
    starts = np.flatnonzero(boundary)
    key = key[starts]
    return (
        key // span_output + base_input,
        key % span_output + base_output,
        np.add.reduceat(values, starts),
    )


def weights_conservative_2d(grid_input, grid_output, weights_input=None, nthreads: int = 0):
    """Coalesced conservative weights of one 2D element (sorted by (input, output))."""
    return coalesce(*sweep_2d(grid_input, grid_output, weights_input, nthreads))


def locate(grid, px, py, method: str = "brute"):
    """``index_of_point_brute`` / ``index_of_point_secant`` (_grids.py:218-463) for many points."""
    x, y = (_f64(a) for a in grid)
    px, py = _f64(px).reshape(-1), _f64(py).reshape(-1)
    oi = np.empty(px.shape, dtype=np.int64)
    oj = np.empty(px.shape, dtype=np.int64)
    _load().orc_locate_many(x.shape[0], x.shape[1], _ptr(x), _ptr(y), px.size, _ptr(px), _ptr(py),
                            0 if method == "brute" else 1, _ptr(oi), _ptr(oj))
    return oi, oj


# --------------------------------------------------------------------------
# apply
# --------------------------------------------------------------------------


def apply(indices_input, indices_output, values, values_input, n_output, values_output=None):
    """``_regrid_from_weights`` (regridding/_regrid/_regrid_from_weights.py:165-182).

    ``values_input`` is (D, n_input); returns (D, n_output) float64, or fills a
    float32 ``values_output`` in place the way numpy does (update in float64,
    store rounded).
    """
    ii = np.ascontiguousarray(indices_input, dtype=np.int64)
    oo = np.ascontiguousarray(indices_output, dtype=np.int64)
    w = _f64(values)
    vin = np.ascontiguousarray(values_input)
    d, n_in = vin.shape
    lib = _load()
    if values_output is not None and values_output.dtype == np.float32:
        assert vin.dtype == np.float32
        lib.orc_apply_f32in_f32out(d, n_in, n_output, w.size, _ptr(ii), _ptr(oo), _ptr(w), _ptr(vin),
                                   _ptr(values_output))
        return values_output
    out = np.empty((d, n_output), dtype=np.float64)
    if vin.dtype == np.float32:
        lib.orc_apply_f32in(d, n_in, n_output, w.size, _ptr(ii), _ptr(oo), _ptr(w), _ptr(vin), _ptr(out))
    else:
        vin = _f64(vin)
        lib.orc_apply_f64(d, n_in, n_output, w.size, _ptr(ii), _ptr(oo), _ptr(w), _ptr(vin), _ptr(out))
    return out


# --------------------------------------------------------------------------
# 1D
# --------------------------------------------------------------------------


def find_indices_1d(x_input, x_output, fill_value=None, method="brute"):
    """``_find_indices_{brute,searchsorted}_1d`` on (D, m) / (D, n) arrays."""
    xi = _f64(x_input)
    xo = _f64(x_output)
    xi2 = xi.reshape(-1, xi.shape[-1])
    xo2 = xo.reshape(-1, xo.shape[-1])
    nd = max(xi2.shape[0], xo2.shape[0])
    si = 0 if xi2.shape[0] == 1 else xi2.shape[1]
    so = 0 if xo2.shape[0] == 1 else xo2.shape[1]
    fill = np.iinfo(np.int64).max if fill_value is None else int(fill_value)
    res = np.empty((nd, xo2.shape[1]), dtype=np.int64)
    fn = _load().orc_find_indices_brute if method == "brute" else _load().orc_find_indices_searchsorted
    fn(nd, xi2.shape[1], _ptr(xi2), si, xo2.shape[1], _ptr(xo2), so, fill, _ptr(res))
    return res


def multilinear_1d(x_input, x_output, weights_input=None, bounds="extrapolate"):
    """``_weights_from_indices_multilinear`` for 1D (regridding/_weights/_weights_multilinear.py:40-206).

    Inputs are already-normalised (D, m) / (D, n) arrays.  Returns a list of D
    uncoalesced (indices_input, indices_output, values) triples.
    """
    xi = _f64(x_input)
    xo = _f64(x_output)
    nd = xo.shape[0]
    index = find_indices_1d(xi, xo, method="searchsorted")
    index_max = xi.shape[-1] - 2
    outside = (index < 0) | (index > index_max)
    if bounds == "raise" and outside.any():
        raise ValueError("output points fall outside the input grid")
    below = xo < xi[..., :1]
    idx = np.ascontiguousarray(np.where(below, 0, np.clip(index, 0, index_max)), dtype=np.int64)
    out_mask = np.ascontiguousarray(outside if bounds == "nan" else np.zeros_like(outside), dtype=np.uint8)
    w = None if weights_input is None else _f64(np.broadcast_to(weights_input, xi.shape))
    n = xo.shape[1]
    ind_in = np.empty((nd, 2 * n), dtype=np.int64)
    ind_out = np.empty((nd, 2 * n), dtype=np.int64)
    val = np.empty((nd, 2 * n), dtype=np.float64)
    si = 0 if xi.shape[0] == 1 else xi.shape[1]
    sw = 0 if (w is None or w.shape[0] == 1) else w.shape[1]
    _load().orc_multilinear_1d(nd, xi.shape[1], _ptr(xi), si, n, _ptr(xo), xo.shape[1], _ptr(idx),
                               _ptr(w), sw, _ptr(out_mask), _ptr(ind_in), _ptr(ind_out), _ptr(val))
    return [(ind_in[d], ind_out[d], val[d]) for d in range(nd)]


def conservative_1d(x_input, x_output, weights_input=None):
    """``_weights_conservative_1d`` (regridding/_weights/_weights_conservative_1d/_weights_conservative_1d.py:59-189)."""
    xi = _f64(x_input)
    xo = _f64(x_output)
    w = None if weights_input is None else _f64(weights_input)
    cap = 2 * (xi.size + xo.size) + 8
    ind_in = np.empty(cap, dtype=np.int64)
    ind_out = np.empty(cap, dtype=np.int64)
    val = np.empty(cap, dtype=np.float64)
    work = np.empty(xi.size + xo.size + xi.size, dtype=np.float64)
    n = _load().orc_conservative_1d(xi.size, _ptr(xi), xo.size, _ptr(xo), _ptr(w), cap, _ptr(ind_in),
                                    _ptr(ind_out), _ptr(val), _ptr(work))
    if n < 0:
        raise RuntimeError("oracle conservative_1d capacity exceeded")
    return ind_in[:n].copy(), ind_out[:n].copy(), val[:n].copy()


def ndarray_linear_interpolation(a, indices, axis=None, axis_indices=None):
    """``ndarray_linear_interpolation`` (regridding/_interp_ndarray.py:11-223):
    the axis bookkeeping of :66-163 and the point formulas of
    ``_linear_interpolation`` (:192-217) and ``_bilinear_interpolation``
    (:220-268), vectorised with numpy in the same operation order (one
    rounding per operation, as the pure-Python evaluation does)."""
    a = np.asarray(a)
    ndim_a = a.ndim
    b = np.broadcast(*indices)
    shape_i, ndim_i = b.shape, b.ndim
    if axis is None:
        axis = tuple(range(ndim_a))
    axis = np.lib.array_utils.normalize_axis_tuple(axis, ndim=ndim_a)
    axis = tuple(int(v) for v in ~(~np.array(axis) % ndim_a))
    if axis_indices is None:
        axis_indices = tuple(range(ndim_i))
    axis_indices = np.lib.array_utils.normalize_axis_tuple(axis_indices, ndim=ndim_i)
    axis_indices = tuple(int(v) for v in ~(~np.array(axis_indices) % ndim_i))
    if len(indices) != len(axis):
        raise ValueError("number of indices must match the number of axes")
    orth_a = tuple(ax for ax in range(-ndim_a, 0) if ax not in axis)
    orth_i = tuple(ax for ax in range(-ndim_i, 0) if ax not in axis_indices)
    shape_orth = np.broadcast_shapes(tuple(a.shape[ax] for ax in orth_a), tuple(shape_i[ax] for ax in orth_i))
    nba, nbi = len(shape_orth) + len(axis), len(shape_orth) + len(axis_indices)
    shape_ba = tuple(a.shape[ax] if ax in axis else shape_orth[orth_a.index(ax)] for ax in range(-nba, 0))
    shape_bi = tuple(shape_i[ax] if ax in axis_indices else shape_orth[orth_i.index(ax)] for ax in range(-nbi, 0))
    a = np.broadcast_to(a, shape_ba)
    idx = tuple(np.broadcast_to(i, shape_bi) for i in indices)
    result = np.empty(shape_bi)
    for index in np.ndindex(*shape_orth):
        ia = tuple(slice(None) if ax in axis else index[orth_a.index(ax)] for ax in range(-nba, 0))
        ii = tuple(slice(None) if ax in axis_indices else index[orth_i.index(ax)] for ax in range(-nbi, 0))
        s = a[ia]
        if len(axis) == 1:
            x = idx[0][ii].reshape(-1).astype(float)
            x0 = np.clip(np.floor(x).astype(np.int64), 0, s.shape[0] - 2)
            dx = x - x0
            r = s[x0] * (1 - dx) + s[x0 + 1] * dx
        elif len(axis) == 2:
            x = idx[0][ii].reshape(-1).astype(float)
            y = idx[1][ii].reshape(-1).astype(float)
            x0 = np.clip(np.floor(x).astype(np.int64), 0, s.shape[0] - 2)
            y0 = np.clip(np.floor(y).astype(np.int64), 0, s.shape[1] - 2)
            dx, dy = x - x0, y - y0
            w00, w01 = (1 - dx) * (1 - dy), (1 - dx) * dy
            w10, w11 = dx * (1 - dy), dx * dy
            r = (s[x0, y0] * w00) + (s[x0, y0 + 1] * w01) + (s[x0 + 1, y0] * w10) + (s[x0 + 1, y0 + 1] * w11)
        else:
            raise NotImplementedError
        result[ii] = r.reshape(idx[0][ii].shape)
    return result


# --------------------------------------------------------------------------
# fill (red-black Gauss-Seidel)
# --------------------------------------------------------------------------


def fill_median_guess(a: np.ndarray, where: np.ndarray, axis: tuple[int, ...]) -> np.ndarray:
    """``_guess_median`` (regridding/_fill/_gauss_seidel.py:61-80): the
    median of the valid elements along ``axis``, 0 where there are none."""
    import warnings

    b = np.where(where, np.nan, a)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", category=RuntimeWarning)
        med = np.nanmedian(b, axis=axis, keepdims=True)
    return np.where(np.isnan(med), 0, med)


def fill(a, where=None, axis=None, guess=None, num_iterations: int = 100) -> np.ndarray:
    """``fill(method="gauss_seidel")`` (regridding/_fill/_fill.py:10-109,
    _gauss_seidel.py:12-58): the host steps in numpy, the sweeps in C
    (``orc_fill_gauss_seidel_f64``; float32 arrays follow Numba's typing in
    ``orc_fill_gauss_seidel_f32``)."""
    if where is None:
        where = np.isnan(a)
    a = np.array(a, copy=True)
    a, where = np.broadcast_arrays(a, where, subok=True)
    a = np.array(a)
    ndim = a.ndim
    axis = tuple(range(ndim)) if axis is None else axis
    axis = np.lib.array_utils.normalize_axis_tuple(axis, ndim=ndim)
    axis = tuple(int(v) for v in ~(~np.array(axis) % ndim))
    if guess is None:
        guess = fill_median_guess(a, where, axis)
    a[where] = np.broadcast_to(guess, a.shape)[where]
    if len(axis) != 2:
        raise ValueError(f"The number of interpolation axes, {len(axis)},is not supported")
    dest = (-2, -1)
    shape_slice = tuple(a.shape[ax] for ax in axis)
    moved = np.moveaxis(a, axis, dest)
    shape_moved = moved.shape
    work = np.ascontiguousarray(moved.reshape(-1, *shape_slice))
    w = np.ascontiguousarray(np.moveaxis(where, axis, dest).reshape(-1, *shape_slice), dtype=np.uint8)
    nt, ny, nx = work.shape
    if num_iterations > 0 and nt > 0 and (nx == 1 or ny == 1):
        raise ZeroDivisionError("float division by zero")
    if work.dtype == np.float32:
        _load().orc_fill_gauss_seidel_f32(nt, ny, nx, _ptr(work), _ptr(w), int(num_iterations))
    else:
        work = work.astype(np.float64, copy=False)
        _load().orc_fill_gauss_seidel_f64(nt, ny, nx, _ptr(work), _ptr(w), int(num_iterations))
    return np.moveaxis(work.reshape(shape_moved), dest, axis)

