"""``fill()``: replace the missing elements of an array by red-black
Gauss-Seidel relaxation over two of its axes.

Drop-in for ``regridding.fill`` (regridding/_fill/_fill.py:10-109) and its
Gauss-Seidel method (regridding/_fill/_gauss_seidel.py:12-58): the same
defaults (``where=isnan(a)``, all axes, ``guess`` = the median of the valid
elements of each slice, 100 iterations), axis handling and errors.  The
median, the seeding of the missing elements and every relaxation sweep run on
the GPU (``rg_fill_gauss_seidel``); float64 results are bit-identical to the
upstream's sequential sweep.  float32 arrays are relaxed with Numba's typing
(float32 neighbour sums, float64 products, float32 result); other dtypes are
relaxed in float64 and returned as float64.
"""

from __future__ import annotations

from typing import Literal, Sequence

import numpy as np

from . import _device, _lib, _util

__all__ = ["fill"]


def fill(
    a: np.ndarray,
    where: None | np.ndarray = None,
    axis: None | int | Sequence[int] = None,
    method: Literal["gauss_seidel"] = "gauss_seidel",
    **kwargs,
) -> np.ndarray:
    """Fill the elements of ``a`` selected by ``where`` (default: the NaNs)
    by interpolating from the others along ``axis`` (two axes; default all
    axes of a 2D array).  ``method="gauss_seidel"`` takes ``guess`` (the
    starting value of the missing elements, a scalar or an array
    broadcastable against ``a``; default the median of the valid elements of
    each slice) and ``num_iterations`` (default 100)."""
    if where is None:
        where = np.isnan(a)
    if method == "gauss_seidel":
        return fill_gauss_seidel(a=a, where=where, axis=axis, **kwargs)
    raise ValueError(f"Unrecognized method '{method}'")


def _plan(a, where, axis, guess):
    """Broadcast, axis normalisation and the moved (nt, ny, nx) layout of
    _gauss_seidel.py:21-48, with the guess as one value per slice when it is
    constant over the two axes, else one per cell."""
    a = np.asarray(a)
    a, where = np.broadcast_arrays(a, np.asarray(where), subok=True)
    if a.dtype not in (np.float32, np.float64):
        a = a.astype(np.float64)
    axis = _util.normalize_axis(axis, a.ndim)
    if len(axis) != 2:
        raise ValueError(f"The number of interpolation axes, {len(axis)},is not supported")
    dest = (-2, -1)
    moved_shape = np.moveaxis(a, axis, dest).shape
    ny, nx = moved_shape[-2:]
    nt = int(np.prod(moved_shape[:-2], dtype=np.int64))
    rows = np.ascontiguousarray(np.moveaxis(a, axis, dest)).reshape(nt, ny, nx)
    mask = np.ascontiguousarray(np.moveaxis(where.astype(bool, copy=False), axis, dest)).reshape(nt, ny, nx)
    if guess is None:
        kind, g = _lib.RG_FILL_GUESS_MEDIAN, None
    else:
        gb = np.moveaxis(np.broadcast_to(np.asarray(guess), a.shape), axis, dest)
        if all(gb.shape[d] == 1 or gb.strides[d] == 0 for d in (-2, -1)):
            kind, g = _lib.RG_FILL_GUESS_SLICE, np.ascontiguousarray(gb[..., 0, 0].reshape(nt), dtype=a.dtype)
        else:
            kind, g = _lib.RG_FILL_GUESS_FULL, np.ascontiguousarray(gb.reshape(nt, ny, nx), dtype=a.dtype)
    return rows, mask.view(np.uint8), kind, g, axis, moved_shape


def fill_gauss_seidel(
    a: np.ndarray,
    where: np.ndarray,
    axis: None | int | Sequence[int],
    guess: None | float | np.ndarray = None,
    num_iterations: int = 100,
) -> np.ndarray:
    """The Gauss-Seidel method of :func:`fill` (regridding/_fill/_gauss_seidel.py:12-58)."""
    rows, mask, kind, g, axis, moved_shape = _plan(a, where, axis, guess)
    nt, ny, nx = rows.shape
    num_iterations = int(num_iterations)
    if num_iterations > 0 and nt > 0 and (nx == 1 or ny == 1):
        raise ZeroDivisionError("float division by zero")
    if rows.size:
        d_a = _device.upload(rows)
        d_w = _device.upload(mask)
        d_g = None if g is None else _device.upload(g)
        dtype = _lib.RG_F64 if rows.dtype == np.float64 else _lib.RG_F32
        _lib.call("rg_fill_gauss_seidel", _device.ptr(d_a), dtype, _device.ptr(d_w), nt, ny, nx, _device.ptr(d_g),
                  kind, max(num_iterations, 0), _device.stream())
        rows = _device.download(d_a)
    return np.moveaxis(rows.reshape(moved_shape), (-2, -1), axis)
