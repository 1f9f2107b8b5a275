"""``weights()``: build the sparse regridding matrix on the GPU.

Host-side structure follows regridding/_weights/_weights.py:13-196,
regridding/_weights/_weights_conservative.py:11-146 and
regridding/_weights/_weights_multilinear.py:9-139; the per-element work runs
in ``libregrid_gb300.so``.
"""

from __future__ import annotations

import ctypes
from typing import Literal, Sequence

import numpy as np

from . import _device, _lib, _util

__all__ = ["weights"]


def weights(
    coordinates_input: tuple[np.ndarray, ...],
    coordinates_output: tuple[np.ndarray, ...],
    axis_input: None | int | Sequence[int] = None,
    axis_output: None | int | Sequence[int] = None,
    weights_input: None | np.ndarray = None,
    method: Literal["multilinear", "conservative"] = "multilinear",
    bounds: Literal["extrapolate", "nan", "raise"] = "extrapolate",
    perturb: None | bool = None,
    seed: "None | int | np.random.Generator" = _util.SEED_DEFAULT,
) -> tuple[np.ndarray, tuple[int, ...], tuple[int, ...]]:
    """Save a regridding operation as sparse weights (drop-in for ``regridding.weights``).

    Returns ``(weights, shape_input, shape_output)`` where ``weights`` is an
    object array over the orthogonal (not resampled) axes whose elements are
    ``(indices_input, indices_output, values)`` flat arrays (int64, int64,
    float64) with unique ``(input, output)`` pairs sorted by input then
    output.  The arrays are read-only: the library keeps a device copy of the
    matrix keyed by them, which :func:`regridding_gb300.regrid_from_weights`
    reuses.  ``method``, ``bounds``, ``perturb`` and ``seed`` have the
    upstream meanings; the seeded perturbation of the output grid is drawn on
    the host with the same generator calls, so results are reproducible and
    identical to the upstream package's for the same seed.
    """
    array, shape_in, shape_out, _ = _weights_device(
        coordinates_input, coordinates_output, axis_input, axis_output, weights_input, method, bounds,
        perturb, seed, want_host=True)
    return array, shape_in, shape_out


def _weights_device(coordinates_input, coordinates_output, axis_input, axis_output, weights_input, method,
                    bounds, perturb, seed, want_host: bool):
    """Build and return ``(array, shape_input, shape_output, device)`` where
    ``device`` lists a :class:`DeviceWeights` per flat element (or None)."""
    unit_weights = getattr(weights_input, "unit", None)
    if unit_weights is not None:
        weights_input = getattr(weights_input, "value")

    if method == "multilinear":
        array, shape_in, shape_out, dev = _multilinear(
            coordinates_input, coordinates_output, axis_input, axis_output, weights_input, bounds, perturb,
            seed)
    elif method == "conservative":
        array, shape_in, shape_out, dev = _conservative(
            coordinates_input, coordinates_output, axis_input, axis_output, weights_input, perturb, seed,
            want_host)
    else:
        raise ValueError(f"unrecognized method '{method}'")

    if unit_weights is not None and array is not None:
        flat = array.reshape(-1)
        for k in range(flat.size):
            ii, oo, vv = flat[k]
            flat[k] = (ii, oo, vv << unit_weights)
    return array, shape_in, shape_out, dev


def _elements(nd: int, h_in, h_out, h_val, counts) -> np.ndarray:
    """The saved layout's elements as views of the first ``counts[d]``
    entries of row ``d`` of the downloaded (nd, cap) arrays: no per-element
    copy (10^5 spectra of ~1,800 entries are 4.3 GB).  Writable, as the
    upstream's arrays are."""
    flat = np.empty(nd, dtype=object)
    for d, c in enumerate(counts):
        flat[d] = (h_in[d, :c], h_out[d, :c], h_val[d, :c])
    return flat


def _rows(a: np.ndarray, axes, last: int):
    """Move ``axes`` last and flatten the rest into rows: ``(rows, stride)``.

    When every row is the same broadcast row, one row is returned with a
    stride of 0 so the device reads it for all rows without a copy.
    """
    moved = np.moveaxis(a, axes, _util.numba_axes(len(axes)) if len(axes) > 1 else ~0)
    lead = moved.shape[: moved.ndim - len(axes)]
    nrows = int(np.prod(lead)) if lead else 1
    if nrows > 1 and all(s == 0 for s in moved.strides[: len(lead)]):
        one = np.ascontiguousarray(moved[(0,) * len(lead)]).reshape(1, last)
        return one, 0, nrows
    return np.ascontiguousarray(moved).reshape(nrows, last), last, nrows


# ---------------------------------------------------------------------------
# conservative
# ---------------------------------------------------------------------------


def _conservative(ci, co, axis_input, axis_output, weights_input, perturb, seed, want_host):
    if perturb is None:
        perturb = not isinstance(ci, np.ndarray) and len(ci) > 1

    ci, co, axi, axo, shape_in, shape_out, shape_orth = _util.normalize_input_output_coordinates(
        ci, co, axis_input, axis_output, perturb=perturb, seed=seed)

    shape_values_input = list(shape_in)
    for ax in axi:
        shape_values_input[ax] -= 1
    shape_values_input = tuple(shape_values_input)
    shape_values_output = list(shape_out)
    for ax in axo:
        shape_values_output[ax] -= 1
    shape_values_output = tuple(shape_values_output)

    if weights_input is not None:
        weights_input = np.broadcast_to(weights_input, shape_values_input)

    if len(axi) == 1:
        array, dev = _conservative_1d(ci[0], co[0], axi, axo, weights_input, shape_orth)
        return array, shape_values_input, shape_values_output, dev

    array = np.empty(shape_orth, dtype=object)
    dev = []
    for index in np.ndindex(*shape_orth):
        if len(axi) != 2:
            raise NotImplementedError("Regridding operations greater than 2D are not supported")
        sel_in = list(reversed(index))
        for ax in axi:
            sel_in.insert(~ax, slice(None))
        sel_in = tuple(reversed(sel_in))
        sel_out = list(reversed(index))
        for ax in axo:
            sel_out.insert(~ax, slice(None))
        sel_out = tuple(reversed(sel_out))
        # the upstream indexes the broadcast weights by the orthogonal index
        # directly (_weights_conservative.py:125-126)
        w_index = None if weights_input is None else weights_input[index]
        dw = _device.build_conservative_2d(
            (np.ascontiguousarray(ci[0][sel_in], dtype=float), np.ascontiguousarray(ci[1][sel_in], dtype=float)),
            (np.ascontiguousarray(co[0][sel_out], dtype=float), np.ascontiguousarray(co[1][sel_out], dtype=float)),
            None if w_index is None else np.ascontiguousarray(w_index, dtype=float),
        )
        if want_host:
            element = tuple(dw.export_numpy())
            _device.remember(element, dw)
            array[index] = element
        dev.append(dw)
    return (array if want_host else None), shape_values_input, shape_values_output, dev


def _conservative_1d(x_in, x_out, axi, axo, weights_input, shape_orth):
    m = x_in.shape[axi[0]]
    n = x_out.shape[axo[0]]
    xi, si, nd = _rows(x_in, axi, m)
    xo, so, nd_o = _rows(x_out, axo, n)
    nd = max(nd, nd_o)
    wi, sw = None, 0
    if weights_input is not None:
        wi, sw, _ = _rows(weights_input, axi, m - 1)
        wi = np.asarray(wi, dtype=float)
    t = _device.torch()
    cap = m + n + 2
    d_xi = _device.upload(xi, np.float64)
    d_xo = _device.upload(xo, np.float64)
    d_wi = None if wi is None else _device.upload(wi, np.float64)
    ind_in = t.empty((nd, cap), dtype=t.int64, device="cuda")
    ind_out = t.empty((nd, cap), dtype=t.int64, device="cuda")
    val = t.empty((nd, cap), dtype=t.float64, device="cuda")
    count = t.empty(nd, dtype=t.int64, device="cuda")
    _lib.call("rg_conservative_1d", _device.ptr(d_xi), si, m, _device.ptr(d_xo), so, n, nd, _device.ptr(d_wi),
              sw, cap, _device.ptr(ind_in), _device.ptr(ind_out), _device.ptr(val), _device.ptr(count),
              _device.stream())
    h_in, h_out, h_val, h_cnt = (_device.download(a) for a in (ind_in, ind_out, val, count))
    return _elements(nd, h_in, h_out, h_val, h_cnt.tolist()).reshape(shape_orth), [None] * nd


# ---------------------------------------------------------------------------
# multilinear
# ---------------------------------------------------------------------------


def _multilinear(ci, co, axis_input, axis_output, weights_input, bounds, perturb, seed):
    # the cell search (find_indices, searchsorted) sees unperturbed coordinates
    ci_s, co_s, axi_s, axo_s, *_ = _util.normalize_input_output_coordinates(ci, co, axis_input, axis_output)
    if len(axi_s) != 1:
        raise ValueError(f"{len(axi_s)}-dimensional searchsorted not supported")
    if bounds not in ("extrapolate", "nan", "raise"):
        raise ValueError(f"Unrecognized {bounds=}, expected one of ('extrapolate', 'nan', 'raise').")
    if perturb is None:
        perturb = False
    ci_n, co_n, axi, axo, shape_in, shape_out, shape_orth = _util.normalize_input_output_coordinates(
        ci, co, axis_input, axis_output, perturb=perturb, seed=seed)

    m = shape_in[axi[0]]
    n = shape_out[axo[0]]
    xi, si, nd_i = _rows(ci_n[0], axi, m)
    xo, so, nd = _rows(co_n[0], axo, n)
    xs = None
    if perturb:
        xs, so_s, _ = _rows(co_s[0], axo_s, n)
        if so_s != so:
            xs = np.ascontiguousarray(np.broadcast_to(xs, xo.shape))
    nd = max(nd, nd_i)
    if so == 0 and nd > 1:
        # every row has the same output points but the weights are per row
        xo = np.ascontiguousarray(np.broadcast_to(xo, (nd, n)))
        so = n
        if xs is not None:
            xs = np.ascontiguousarray(np.broadcast_to(xs, (nd, n)))
    wi, sw = None, 0
    if weights_input is not None:
        wi, sw, _ = _rows(np.broadcast_to(weights_input, shape_in), axi, m)
        wi = np.asarray(wi, dtype=float)

    t = _device.torch()
    d_xi = _device.upload(xi, np.float64)
    d_xo = _device.upload(xo, np.float64)
    d_xs = None if xs is None else _device.upload(xs, np.float64)
    d_wi = None if wi is None else _device.upload(wi, np.float64)
    ind_in = t.empty((nd, 2 * n), dtype=t.int64, device="cuda")
    ind_out = t.empty((nd, 2 * n), dtype=t.int64, device="cuda")
    val = t.empty((nd, 2 * n), dtype=t.float64, device="cuda")
    n_out = ctypes.c_int64(0)
    _lib.call("rg_multilinear_1d", _device.ptr(d_xi), si, m, _device.ptr(d_xo), _device.ptr(d_xs), so, n, nd,
              _device.ptr(d_wi), sw, _lib.RG_BOUNDS[bounds], _device.ptr(ind_in), _device.ptr(ind_out),
              _device.ptr(val), ctypes.byref(n_out) if bounds == "raise" else None, _device.stream())
    if bounds == "raise" and n_out.value:
        raise ValueError(
            f"{n_out.value} of the output points fall outside the input grid, and {bounds=}.")
    h_in, h_out, h_val = (_device.download(a) for a in (ind_in, ind_out, val))
    return _elements(nd, h_in, h_out, h_val, [h_in.shape[1]] * nd).reshape(shape_orth), shape_in, shape_out, \
        [None] * nd
