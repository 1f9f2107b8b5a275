"""``transpose_weights()`` and ``transpose_weights_conservative()``.

Follow regridding/_weights/_weights_transposed/_weights_transposed.py:13-340;
cell volumes and the conservative rescaling run on the GPU.
"""

from __future__ import annotations

import numpy as np

from . import _device, _lib, _util

__all__ = ["transpose_weights", "transpose_weights_conservative"]


def transpose_weights(weights):
    """Swap the index arrays of every element, without copying (drop-in for
    ``regridding.transpose_weights``): ``(i, j, w) -> (j, i, w)``."""
    array, shape_input, shape_output = weights
    shape = array.shape
    flat = array.reshape(-1)
    result = np.empty(flat.size, dtype=object)
    for d in range(flat.size):
        ii, oo, vv = flat[d]
        result[d] = (oo, ii, vv)
    return result.reshape(shape), shape_output, shape_input


def cell_volume(grid: tuple[np.ndarray, ...], axis: tuple[int, ...]) -> np.ndarray:
    """Cell lengths (1D) or areas (2D) of each grid along ``axis`` (ascending),
    computed on the GPU (``_cell_volume``, _weights_transposed.py:262-340)."""
    shape = grid[0].shape
    numba = _util.numba_axes(len(axis))
    shape_numba = tuple(shape[ax] for ax in axis)
    t = _device.torch()
    if len(grid) == 1:
        (x,) = grid
        xr = np.moveaxis(x, axis, numba).reshape((-1,) + shape_numba)
        d_x = _device.upload(xr, np.float64)
        nd, n = xr.shape
        out = t.empty((nd, n - 1), dtype=t.float64, device="cuda")
        _lib.call("rg_cell_length_1d", _device.ptr(d_x), nd, n, _device.ptr(out), _device.stream())
        res = _device.download(out)
        res = res.reshape(xr.shape[:-1] + res.shape[-1:])
        return np.moveaxis(res, numba, axis)
    if len(grid) == 2:
        x, y = grid
        xr = np.moveaxis(x, axis, numba).reshape((-1,) + shape_numba)
        yr = np.moveaxis(y, axis, numba).reshape((-1,) + shape_numba)
        nd, nx, ny = xr.shape
        res = np.empty((nd, nx - 1, ny - 1))
        for d in range(nd):
            d_x = _device.upload(xr[d], np.float64)
            d_y = _device.upload(yr[d], np.float64)
            out = t.empty((nx - 1, ny - 1), dtype=t.float64, device="cuda")
            _lib.call("rg_cell_area_2d", _device.ptr(d_x), _device.ptr(d_y), nx, ny, _device.ptr(out),
                      _device.stream())
            res[d] = _device.download(out)
        res = res.reshape(xr.shape[:-2] + res.shape[-2:])
        return np.moveaxis(res, numba, axis)
    raise ValueError("Grids greater than 2D not supported.")


def transpose_weights_conservative(
    weights,
    coordinates_input,
    coordinates_output,
    axis_input=None,
    axis_output=None,
    weights_input=None,
):
    """Conservative transpose (drop-in for ``regridding.transpose_weights_conservative``):
    each weight becomes ``w * vol_in[i] / vol_out[o]`` (divided first by
    ``weights_input[i]**2`` when given) and the index arrays are swapped."""
    weights_array, shape_input, shape_output = weights
    ci, co, axi, axo, _, _, shape_orth = _util.normalize_input_output_coordinates(
        coordinates_input, coordinates_output, axis_input, axis_output)
    axi = tuple(sorted(axi))
    axo = tuple(sorted(axo))
    numba_in = _util.numba_axes(len(axi))
    numba_out = _util.numba_axes(len(axo))
    size_orth = int(np.prod(shape_orth))

    if weights_input is not None:
        weights_input = np.broadcast_to(weights_input, shape_input)
        weights_input = np.moveaxis(weights_input, axi, numba_in).reshape(size_orth, -1)

    vol_in = np.moveaxis(cell_volume(ci, axi), axi, numba_in).reshape(size_orth, -1)
    vol_out = np.moveaxis(cell_volume(co, axo), axo, numba_out).reshape(size_orth, -1)

    t = _device.torch()
    shape = weights_array.shape
    flat = weights_array.reshape(-1)
    result = np.empty(flat.size, dtype=object)
    for d in range(flat.size):
        ii, oo, vv = flat[d]
        vv = np.asarray(getattr(vv, "value", vv), dtype=np.float64)
        d_ii = _device.upload(np.asarray(ii), np.int64)
        d_oo = _device.upload(np.asarray(oo), np.int64)
        d_vv = _device.upload(vv, np.float64)
        d_vi = _device.upload(vol_in[d], np.float64)
        d_vo = _device.upload(vol_out[d], np.float64)
        d_wi = None if weights_input is None else _device.upload(weights_input[d], np.float64)
        out = t.empty(vv.shape[0], dtype=t.float64, device="cuda")
        _lib.call("rg_transpose_conservative_scale", _device.ptr(d_ii), _device.ptr(d_oo), _device.ptr(d_vv),
                  vv.shape[0], _device.ptr(d_vi), vol_in[d].size, _device.ptr(d_vo), vol_out[d].size,
                  _device.ptr(d_wi), _device.ptr(out), _device.stream())
        result[d] = (oo, ii, _device.download(out))
    return result.reshape(shape), shape_output, shape_input
