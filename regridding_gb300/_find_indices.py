"""``find_indices()``: the cell of the input grid containing each output vertex.

Host-side structure follows regridding/_find_indices/_find_indices.py:12-136.
1D searches run on the GPU with the upstream semantics bit for bit.  2D
(curvilinear) grids, which the upstream rejects, are supported as an
extension: ``method="brute"`` returns the lowest-index containing cell (the
answer of the upstream's internal index_of_point_brute,
regridding/_weights/_weights_conservative_2d/_grids.py:218-279) found by a
GPU grid walk; ``method="exhaustive"`` scans all cells in that order.
"""

from __future__ import annotations

from typing import Literal, Sequence

import numpy as np

from . import _device, _lib, _util

__all__ = ["find_indices"]


def find_indices(
    coordinates_input: tuple[np.ndarray, ...],
    coordinates_output: tuple[np.ndarray, ...],
    axis_input: None | int | Sequence[int] = None,
    axis_output: None | int | Sequence[int] = None,
    fill_value: None | int = None,
    method: Literal["brute", "searchsorted"] = "brute",
) -> tuple[np.ndarray, ...]:
    """Index of the input cell containing each output vertex (drop-in for
    ``regridding.find_indices``); points outside get ``fill_value``
    (default ``numpy.iinfo(int).max``)."""
    ci, co, axi, axo, shape_in, shape_out, shape_orth = _util.normalize_input_output_coordinates(
        coordinates_input, coordinates_output, axis_input, axis_output)
    if fill_value is None:
        fill_value = np.iinfo(int).max

    if len(axi) == 2:
        # 2D: keep the resampled axes in ascending order, so (i, j) index the
        # grid as stored (the upstream has no 2D search to follow here)
        axi, axo = tuple(sorted(axi)), tuple(sorted(axo))
    numba_in = _util.numba_axes(len(axi))
    numba_out = _util.numba_axes(len(axo))
    shape_in_numba = tuple(shape_in[ax] for ax in axi)
    shape_out_numba = tuple(shape_out[ax] for ax in axo)
    ci = tuple(np.moveaxis(v, axi, numba_in).reshape(-1, *shape_in_numba) for v in ci)
    co = tuple(np.moveaxis(v, axo, numba_out).reshape(-1, *shape_out_numba) for v in co)

    # "exhaustive" exists only for the 2D extension; in 1D the upstream knows
    # "brute" and "searchsorted" and rejects every other name
    # (regridding/_find_indices/_find_indices.py:112-125)
    if method not in ("brute", "searchsorted", "exhaustive") or (method == "exhaustive" and len(ci) == 1):
        raise ValueError(f"method `{method}` not recognized.")

    if len(ci) == 1:
        result = (_find_1d(ci[0], co[0], int(fill_value), method),)
    elif len(ci) == 2:
        if method == "searchsorted":
            raise ValueError("2-dimensional searchsorted not supported")
        result = _find_2d(ci, co, int(fill_value), method)
    else:
        raise ValueError(f"{len(ci)}-dimensional brute-force search not supported")

    return tuple(
        np.moveaxis(a.reshape(*shape_orth, *shape_out_numba), source=numba_out, destination=axo) for a in result
    )


def _find_1d(x_in: np.ndarray, x_out: np.ndarray, fill: int, method: str) -> np.ndarray:
    t = _device.torch()
    nd = max(x_in.shape[0], x_out.shape[0])
    m = x_in.shape[1]
    n = x_out.shape[1]
    d_in = _device.upload(x_in, np.float64)
    d_out = _device.upload(x_out, np.float64)
    res = t.empty((nd, n), dtype=t.int64, device="cuda")
    _lib.call("rg_find_indices_1d", _device.ptr(d_in), m if x_in.shape[0] > 1 else 0, m, _device.ptr(d_out),
              n if x_out.shape[0] > 1 else 0, n, nd, 0 if method == "brute" else 1, fill, _device.ptr(res),
              _device.stream())
    return _device.download(res)


def locate_2d(grid, px, py, method: str = "brute"):
    """Cell (i, j) of a 2D vertex grid containing each point; ``(INT64_MAX,
    INT64_MAX)`` outside.  ``method``: "brute" (grid walk, lowest-index
    containing cell), "exhaustive" (upstream brute order), "secant" (the
    upstream secant locator).  Inputs and outputs are numpy arrays or CUDA
    tensors."""
    t = _device.torch()
    x, y = (g if isinstance(g, t.Tensor) else _device.upload(np.asarray(g), np.float64) for g in grid)
    x = x.to(t.float64).contiguous()
    y = y.to(t.float64).contiguous()
    is_tensor = isinstance(px, t.Tensor)
    dpx = px.to(t.float64).contiguous().reshape(-1) if is_tensor else _device.upload(np.ravel(px), np.float64)
    dpy = py.to(t.float64).contiguous().reshape(-1) if is_tensor else _device.upload(np.ravel(py), np.float64)
    n = dpx.numel()
    oi = t.empty(n, dtype=t.int64, device="cuda")
    oj = t.empty(n, dtype=t.int64, device="cuda")
    code = {"exhaustive": 0, "secant": 1, "brute": 2}[method]
    _lib.call("rg_locate_2d", _device.ptr(x), _device.ptr(y), x.shape[0], x.shape[1], _device.ptr(dpx),
              _device.ptr(dpy), n, code, _device.ptr(oi), _device.ptr(oj), _device.stream())
    if is_tensor:
        return oi, oj
    return _device.download(oi), _device.download(oj)


def _find_2d(ci, co, fill: int, method: str):
    nd = max(ci[0].shape[0], co[0].shape[0])
    n_pts = co[0].shape[1] * co[0].shape[2]
    res_i = np.empty((nd, n_pts), dtype=np.int64)
    res_j = np.empty((nd, n_pts), dtype=np.int64)
    for d in range(nd):
        gx = ci[0][min(d, ci[0].shape[0] - 1)]
        gy = ci[1][min(d, ci[1].shape[0] - 1)]
        px = co[0][min(d, co[0].shape[0] - 1)]
        py = co[1][min(d, co[1].shape[0] - 1)]
        oi, oj = locate_2d((gx, gy), px, py, method=method)
        outside = oi == np.iinfo(np.int64).max
        oi[outside] = fill
        oj[outside] = fill
        res_i[d] = oi
        res_j[d] = oj
    return res_i, res_j
