"""``ndarray_linear_interpolation()``: linear / bilinear interpolation of an
array at fractional indices along one or two of its axes.

Drop-in for ``regridding.ndarray_linear_interpolation``
(regridding/_interp_ndarray.py:11-166): the same axis normalisation, the same
broadcasting of the orthogonal axes of ``a`` against those of the indices,
and a float64 result shaped like the broadcast indices.  The upstream loops
over the orthogonal elements in Python and evaluates each element's points
in a numba kernel; here every point of every element is one thread of a
single ``rg_interp_linear`` launch, with the upstream per-point operation
order (bit-identical results).
"""

from __future__ import annotations

import numpy as np

from . import _device, _lib

__all__ = ["ndarray_linear_interpolation"]


def _negative_axes(axis, ndim: int) -> tuple[int, ...]:
    """``axis`` as a tuple of negative axis numbers (upstream :77-87)."""
    axis = np.lib.array_utils.normalize_axis_tuple(axis, ndim=ndim)
    return tuple(int(ax) - ndim for ax in axis)


def _shared(arr: np.ndarray, orth: tuple[int, ...]) -> bool:
    """Whether every orthogonal axis of the broadcast ``arr`` repeats one
    element (length 1 or stride 0), so all its rows are the same."""
    return all(arr.shape[ax] == 1 or arr.strides[ax] == 0 for ax in orth)


def _to_rows(arr: np.ndarray, orth: tuple[int, ...], kept: tuple[int, ...], shared: bool) -> tuple[np.ndarray, int]:
    """``arr`` (already broadcast) with its orthogonal axes first and the
    ``kept`` axes last, both in storage order, flattened to
    ``(n_orth, -1)`` with its row stride; ``shared`` keeps only the first
    row and gives a row stride of 0."""
    moved = np.moveaxis(arr, orth + kept, tuple(range(len(orth) + len(kept))))
    inner = int(np.prod([arr.shape[ax] for ax in kept], dtype=np.int64))
    rows = moved.reshape(-1, inner)
    if shared:
        return np.ascontiguousarray(rows[:1], dtype=np.float64), 0
    return np.ascontiguousarray(rows, dtype=np.float64), inner


class _Plan:
    """The launch of one call: ``rows_a`` (``(1 or n_orth, nx * ny)``) with
    ``a_stride``, ``rows_i`` (one ``(1 or n_orth, m)`` array per index) with
    ``i_stride``, and how the ``(n_orth, m)`` result goes back into the
    shape of the broadcast indices."""

    __slots__ = ("rows_a", "a_stride", "nx", "ny", "rows_i", "i_stride", "m", "n_orth", "shape_out", "axes_out")


def _plan(a, indices, axis, axis_indices) -> _Plan:
    """Axis normalisation and broadcasting of the upstream
    (regridding/_interp_ndarray.py:66-131), as the flat rows one launch
    reads."""
    a = np.asarray(a)
    indices = tuple(np.asarray(i) for i in indices)
    shape_i = np.broadcast(*indices).shape
    ndim_a, ndim_i = a.ndim, len(shape_i)

    axis = _negative_axes(tuple(range(ndim_a)) if axis is None else axis, ndim_a)
    axis_indices = _negative_axes(tuple(range(ndim_i)) if axis_indices is None else axis_indices, ndim_i)
    if len(indices) != len(axis):
        raise ValueError(
            f"The number of indices, {len(indices)}, must match the number of elements in axis, {len(axis)}")
    if len(axis) not in (1, 2):
        raise NotImplementedError(f"interpolation along {len(axis)} axes is not supported")

    orth_a = tuple(ax for ax in range(-ndim_a, 0) if ax not in axis)
    orth_i = tuple(ax for ax in range(-ndim_i, 0) if ax not in axis_indices)
    if len(orth_a) != len(orth_i):
        # the upstream pairs the k-th orthogonal axis of ``a`` with the k-th
        # orthogonal axis of the indices and fails when the counts differ
        raise ValueError(f"a has {len(orth_a)} orthogonal axes and the indices {len(orth_i)}; "
                         f"they must have the same number")
    shape_orth = np.broadcast_shapes(tuple(a.shape[ax] for ax in orth_a), tuple(shape_i[ax] for ax in orth_i))
    shape_ba = list(a.shape)
    for k, ax in enumerate(orth_a):
        shape_ba[ax] = shape_orth[k]
    shape_bi = list(shape_i)
    for k, ax in enumerate(orth_i):
        shape_bi[ax] = shape_orth[k]

    interp_a = tuple(sorted(axis))
    sizes = tuple(a.shape[ax] for ax in interp_a)
    if min(sizes) < 2:
        raise ValueError(f"every interpolated axis needs at least 2 samples, got {sizes}")
    kept_i = tuple(sorted(axis_indices))

    p = _Plan()
    p.nx, p.ny = sizes[0], (sizes[1] if len(sizes) == 2 else 0)
    p.n_orth = int(np.prod(shape_orth, dtype=np.int64))
    p.m = int(np.prod([shape_bi[ax] for ax in kept_i], dtype=np.int64))
    p.shape_out = tuple(shape_orth) + tuple(shape_bi[ax] for ax in kept_i)
    p.axes_out = orth_i + kept_i
    p.rows_a, p.a_stride, p.rows_i, p.i_stride = None, 0, [], 0
    if p.n_orth == 0 or p.m == 0:
        return p
    a_b = np.broadcast_to(a, tuple(shape_ba))
    p.rows_a, p.a_stride = _to_rows(a_b, orth_a, interp_a, _shared(a_b, orth_a))
    ind_b = [np.broadcast_to(ind, tuple(shape_bi)) for ind in indices]
    shared_i = all(_shared(b, orth_i) for b in ind_b)
    for b in ind_b:
        r, p.i_stride = _to_rows(b, orth_i, kept_i, shared_i)
        p.rows_i.append(r)
    return p


def _finish(p: _Plan, flat: np.ndarray) -> np.ndarray:
    """The ``(n_orth, m)`` result in the shape of the broadcast indices."""
    return np.moveaxis(flat.reshape(p.shape_out), tuple(range(len(p.shape_out))), p.axes_out)


def ndarray_linear_interpolation(
    a: np.ndarray,
    indices: tuple[np.ndarray, ...],
    axis: None | int | tuple[int, ...] = None,
    axis_indices: None | int | tuple[int, ...] = None,
) -> np.ndarray:
    """Evaluate ``a`` at the fractional ``indices`` along ``axis`` (all axes
    of ``a`` by default) by linear (one axis) or bilinear (two axes)
    interpolation; indices outside ``[0, n - 1]`` extrapolate the first or
    last cell.  ``axis_indices`` names the axes of the (broadcast) indices
    that run over the new points (all of them by default); the remaining
    axes of ``a`` and of the indices broadcast against each other.  With
    two axes, ``indices[0]`` runs along the lower-numbered axis of ``a``."""
    p = _plan(a, indices, axis, axis_indices)
    if p.n_orth == 0 or p.m == 0:
        return _finish(p, np.empty((p.n_orth, p.m)))
    t = _device.torch()
    out = t.empty((p.n_orth, p.m), dtype=t.float64, device="cuda")
    d_a = _device.upload(p.rows_a, np.float64)
    d_i = [_device.upload(r, np.float64) for r in p.rows_i]
    _lib.call("rg_interp_linear", _device.ptr(d_a), p.a_stride, p.nx, p.ny, _device.ptr(d_i[0]),
              _device.ptr(d_i[1]) if len(d_i) == 2 else None, p.i_stride, p.m, p.n_orth, _device.ptr(out),
              _device.stream())
    return _finish(p, _device.download(out))
