"""Host-side argument normalisation shared by the public functions.

These restate the upstream helpers of regridding/_util.py:1-139 with the same
semantics: the same axis conventions (resampled axes are expressed as negative
indices), the same broadcasting rules and error messages, and the same seeded
perturbation of the output grid, drawn with the same numpy Generator calls in
the same order, so that both implementations see bit-identical perturbed
coordinates.
"""

from __future__ import annotations

from typing import Sequence

import numpy as np

SEED_DEFAULT = 42
"""Default seed of the output-grid perturbation (regridding/_util.py:4)."""

EPSILON_PERTURB = 1e-9
"""Standard deviation of the perturbation, as a fraction of the grid extent."""


def normalize_axis(axis: None | int | Sequence[int], ndim: int) -> tuple[int, ...]:
    """Axes as negative indices (``-ndim .. -1``), validated against ``ndim``.

    Follows regridding/_util.py:12-20.
    """
    if axis is None:
        axis = tuple(range(ndim))
    axis = np.lib.array_utils.normalize_axis_tuple(axis, ndim=ndim)
    return tuple(~(~np.array(axis) % ndim))


def insert_resampled(shape_orthogonal: tuple[int, ...], axes: tuple[int, ...], sizes) -> tuple[int, ...]:
    """Rebuild a full shape from the orthogonal shape by inserting, for each
    (negative) axis in ``axes`` in the given order, the size ``sizes[ax]``."""
    rev = list(reversed(shape_orthogonal))
    for ax in axes:
        rev.insert(~ax, sizes[ax])
    return tuple(reversed(rev))


def normalize_input_output_coordinates(
    coordinates_input,
    coordinates_output,
    axis_input=None,
    axis_output=None,
    perturb: bool = False,
    seed=SEED_DEFAULT,
):
    """Broadcast the coordinate arrays and work out the resampled/orthogonal axes.

    Follows regridding/_util.py:23-139.  Returns ``(coordinates_input,
    coordinates_output, axis_input, axis_output, shape_coordinates_input,
    shape_coordinates_output, shape_orthogonal)`` with both axis tuples sorted
    in descending order.
    """
    if isinstance(coordinates_input, np.ndarray):
        coordinates_input = (coordinates_input,)
    if isinstance(coordinates_output, np.ndarray):
        coordinates_output = (coordinates_output,)

    # a unit on the output coordinates is imposed on the input coordinates
    # before they are compared (duck-typed, no astropy dependency)
    converted = []
    for c_in, c_out in zip(coordinates_input, coordinates_output):
        unit = getattr(c_out, "unit", None)
        if unit is not None:
            c_in = c_in << unit
        converted.append(c_in)
    coordinates_input = tuple(converted)

    shape_ci = np.broadcast(*coordinates_input).shape
    shape_co = np.broadcast(*coordinates_output).shape
    ndim_input = len(shape_ci)
    ndim_output = len(shape_co)

    axis_input = tuple(sorted(normalize_axis(axis_input, ndim=ndim_input), reverse=True))
    axis_output = tuple(sorted(normalize_axis(axis_output, ndim=ndim_output), reverse=True))

    if len(axis_output) != len(axis_input):
        raise ValueError(
            f"The number of axes in `axis_output`, {axis_output}, "
            f"must match the number of axes in `axis_input`, {axis_input}"
        )
    if len(coordinates_input) != len(axis_input):
        raise ValueError(
            f"The number of elements in `coordinates_input`, {len(coordinates_input)}, "
            f"should match the number of axes in `axis_input`, {axis_input}"
        )
    if len(coordinates_output) != len(coordinates_input):
        raise ValueError(
            f"The number of elements in `coordinates_output`, {len(coordinates_output)}, "
            f"should match the number of elements in `coordinates_input`, {len(coordinates_input)}"
        )

    orth_in = tuple(ax for ax in normalize_axis(None, ndim_input) if ax not in axis_input)
    orth_out = tuple(ax for ax in normalize_axis(None, ndim_output) if ax not in axis_output)
    shape_orthogonal = np.broadcast_shapes(
        tuple(shape_ci[ax] for ax in orth_in),
        tuple(shape_co[ax] for ax in orth_out),
    )

    shape_input = insert_resampled(shape_orthogonal, axis_input, shape_ci)
    shape_output = insert_resampled(shape_orthogonal, axis_output, shape_co)

    coordinates_input = tuple(np.broadcast_to(c, shape_input) for c in coordinates_input)
    coordinates_output = tuple(np.broadcast_to(c, shape_output) for c in coordinates_output)

    if perturb:
        rng = np.random.default_rng(seed)
        perturbed = []
        for c in coordinates_output:
            ptp = np.ptp(c, axis=axis_output, keepdims=True)
            perturbed.append(rng.normal(c, ptp * EPSILON_PERTURB))
        coordinates_output = tuple(perturbed)

    return (
        coordinates_input,
        coordinates_output,
        axis_input,
        axis_output,
        shape_ci,
        shape_co,
        shape_orthogonal,
    )


def numba_axes(n: int) -> np.ndarray:
    """The trailing axes ``(-n, ..., -1)`` that resampled axes are moved to."""
    return ~np.arange(n)[::-1]
