"""Generate the committed golden fixtures by running the upstream package.

Run from the repository root (needs the upstream source tree, not available on
GPU hosts):

    python tests/golden/make_golden.py [known] [one_dim] [curvilinear] [interp] [fill]

The upstream package is imported in its JIT-disabled pure-Python mode through
``reference_env`` (the mode its own CI exercises).  Each case below restates
the inputs of one upstream known-answer test (file:line given beside it) or
one benchmark configuration, runs the upstream functions on it, and stores
inputs and outputs in ``tests/golden/*.npz``.  Fixtures are loaded with
``tests/golden/fixtures.py``.
"""

from __future__ import annotations

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import reference_env  # noqa: E402

rg = reference_env.import_reference()
from regridding._weights._weights_conservative_2d import _grids  # noqa: E402
from regridding._weights._weights_conservative_2d._weights_conservative_2d import (  # noqa: E402
    weights_conservative_2d,
)
from regridding._util import _normalize_input_output_coordinates  # noqa: E402

DEG = math.pi / 180


class Store:
    """Collects arrays for one .npz file; cases are prefixed ``<name>/``."""

    def __init__(self):
        self.arrays: dict[str, np.ndarray] = {}
        self.meta: dict[str, dict] = {}

    def put(self, case: str, key: str, value):
        self.arrays[f"{case}/{key}"] = np.asarray(value)

    def put_tuple(self, case: str, key: str, values):
        if isinstance(values, np.ndarray):
            values = (values,)
        for k, v in enumerate(values):
            self.put(case, f"{key}_{k}", v)
        self.meta.setdefault(case, {})[f"{key}_len"] = len(values)

    def put_weights(self, case: str, key: str, weights):
        array, shape_input, shape_output = weights
        flat = array.reshape(-1)
        self.meta.setdefault(case, {})[key] = {
            "shape": list(array.shape),
            "shape_input": [int(s) for s in shape_input],
            "shape_output": [int(s) for s in shape_output],
        }
        for k in range(flat.size):
            ii, oo, vv = flat[k]
            self.put(case, f"{key}_{k}_in", ii)
            self.put(case, f"{key}_{k}_out", oo)
            self.put(case, f"{key}_{k}_val", np.asarray(vv))

    def set_meta(self, case: str, **kw):
        self.meta.setdefault(case, {}).update(kw)

    def save(self, name: str):
        path = os.path.join(HERE, name)
        arrays = dict(self.arrays)
        arrays["__meta__"] = np.array(json.dumps(self.meta))
        np.savez_compressed(path, **arrays)
        print(f"wrote {path}: {len(self.meta)} cases, {os.path.getsize(path) / 1e6:.2f} MB")


def none_or(v):
    return None if v is None else np.asarray(v)


# ---------------------------------------------------------------------------
# conservative 2D known answers:
# regridding/_weights/_weights_conservative_2d/_weights_conservative_2d_test.py:16-301
# ---------------------------------------------------------------------------


def conservative_2d_cases():
    box_x = np.linspace(-1, 1, num=2)[..., np.newaxis]
    box_y = np.linspace(-1, 1, num=2)
    x = np.linspace(-1, 1, num=6)[..., np.newaxis]
    y = np.linspace(-1, 1, num=6)
    x2 = np.linspace(-1, 1, num=11)[..., np.newaxis]
    y2 = np.linspace(-1, 1, num=11)
    r = np.random.RandomState(42).uniform(0, 10, size=(5, 5))

    def rot(a):
        return (x * np.cos(a * DEG) - y * np.sin(a * DEG), x * np.sin(a * DEG) + y * np.cos(a * DEG))

    lin3 = (np.linspace(-1, 1, num=3)[..., np.newaxis], np.linspace(-1, 1, num=3))
    lin3b = (np.linspace(-2, 2, num=3)[..., np.newaxis], np.linspace(-2, 2, num=3))
    return [
        ((box_x, box_y), (2 * box_x, 2 * box_y), np.array([[1]]), None, np.array([[1]])),
        ((-box_x, -box_y), (2 * box_x, 2 * box_y), np.array([[1]]), None, np.array([[1]])),
        ((2 * box_x, 2 * box_y), (box_x, box_y), np.array([[1]]), None, np.array([[0.25]])),
        ((box_x, 2 * box_y), (2 * box_x, box_y), np.array([[1]]), None, np.array([[0.5]])),
        ((2 * box_x, box_y), (box_x, 2 * box_y), np.array([[1]]), None, np.array([[0.5]])),
        (lin3, (2 * box_x, 2 * box_y), np.ones((2, 2)), None, np.array([[4]])),
        ((box_x, box_y), lin3b, np.ones((1, 1)), None, np.ones((2, 2)) / 4),
        ((x, y), (x, y), r, None, r),
        (rot(90), (x, y), r, None, np.rot90(r)),
        (rot(180), (x, y), r, None, np.rot90(r, k=2)),
        (rot(270), (x, y), r, None, np.rot90(r, k=3)),
        ((x, y), rot(90), r, None, np.rot90(r, k=-1)),
        ((x, y), (x, y), r, 1, r),
        ((x, y), (x2, y2), np.array(10), 1, np.array(10 / 2 / 2)),
        ((x2, y2), (x, y), np.array(10), 1, np.array(10 * 2 * 2)),
    ]


def gen_conservative_2d(store: Store):
    for k, (ci, co, vi, wi, expected) in enumerate(conservative_2d_cases()):
        case = f"c2d_{k}"
        cox, coy = co
        co = (cox + 1e-6, coy + 1e-6)
        w = rg.weights(coordinates_input=ci, coordinates_output=co, weights_input=wi,
                       method="conservative", perturb=False)
        res = rg.regrid_from_weights(*w, values_input=vi)
        store.put_tuple(case, "ci", ci)
        store.put_tuple(case, "co", co)
        store.put(case, "values_input", vi)
        if wi is not None:
            store.put(case, "weights_input", wi)
        store.put_weights(case, "weights", w)
        store.put(case, "result", res)
        store.put(case, "expected", expected)
        store.set_meta(case, weights_input=wi is not None, perturb=False)


# ---------------------------------------------------------------------------
# saved-weights contract: regridding/_regrid/_tests/test_regrid_from_weights.py:8-161
# and seeds: regridding/_weights/_weights_test.py:5-103
# ---------------------------------------------------------------------------


def gen_layout_and_seed(store: Store):
    x_in = np.linspace(-1, 1, num=11)
    y_in = np.linspace(-1, 1, num=12)
    xb, yb = np.meshgrid(x_in, y_in, indexing="ij")
    angle = 0.2
    xo = xb * np.cos(angle) - yb * np.sin(angle)
    yo = xb * np.sin(angle) + yb * np.cos(angle)
    values = np.random.default_rng(42).random((10, 11))
    w = rg.weights(coordinates_input=(xb, yb), coordinates_output=(xo, yo), method="conservative")
    case = "layout"
    store.put_tuple(case, "ci", (xb, yb))
    store.put_tuple(case, "co", (xo, yo))
    store.put(case, "values_input", values)
    store.put_weights(case, "weights", w)
    store.put(case, "result", rg.regrid_from_weights(*w, values_input=values))
    store.put(case, "regrid", rg.regrid(coordinates_input=(xb, yb), coordinates_output=(xo, yo),
                                        values_input=values, method="conservative"))
    wt = rg.transpose_weights(w)
    store.put_weights(case, "transposed", wt)
    wtc = rg.transpose_weights_conservative(w, coordinates_input=(xb, yb), coordinates_output=(xo, yo))
    store.put_weights(case, "transposed_conservative", wtc)
    vo = rg.regrid_from_weights(*w, values_input=values)
    store.put(case, "roundtrip", rg.regrid_from_weights(*wtc, values_input=vo))

    # seeds (13 x 12 grids): _weights_test.py:5-103
    x_in = np.linspace(-1, 1, num=13)
    y_in = np.linspace(-1, 1, num=12)
    xb, yb = np.meshgrid(x_in, y_in, indexing="ij")
    xo = xb * np.cos(angle) - yb * np.sin(angle)
    yo = xb * np.sin(angle) + yb * np.cos(angle)
    case = "seed"
    store.put_tuple(case, "ci", (xb, yb))
    store.put_tuple(case, "co", (xo, yo))
    for tag, seed in (("default", 42), ("s12345", 12345), ("s0", 0), ("s1", 1)):
        store.put_weights(case, f"w_{tag}", rg.weights(coordinates_input=(xb, yb), coordinates_output=(xo, yo),
                                                       method="conservative", seed=seed))
    store.put_weights(case, "w_gen12345", rg.weights(coordinates_input=(xb, yb), coordinates_output=(xo, yo),
                                                     method="conservative", seed=np.random.default_rng(12345)))
    store.put_weights(case, "w_unperturbed", rg.weights(coordinates_input=(xb, yb), coordinates_output=(xo, yo),
                                                        method="conservative", perturb=False))
    # the perturbed output grid itself: _util.py:121-129
    _, cop, *_ = _normalize_input_output_coordinates((xb, yb), (xo, yo), perturb=True, seed=42)
    store.put_tuple(case, "co_perturbed", cop)


# ---------------------------------------------------------------------------
# 1D: multilinear (_weights_multilinear_test.py:30-149, _weights_test.py:106-158),
# conservative (_weights_conservative_1d_test.py:6-152), find_indices
# (_find_indices/_tests/test_find_indices.py:7-91)
# ---------------------------------------------------------------------------


def gen_1d(store: Store):
    x = np.linspace(-1, 1, num=10)
    y = np.linspace(-1, 1, num=11)
    xb, yb = np.meshgrid(x, y, indexing="ij")
    new_y = np.linspace(-1, 1, num=5)
    new_x = np.linspace(-1, 1, num=6)
    lin11 = np.linspace(-1, 1, num=11)
    ml_cases = [
        ((lin11,), (lin11,), np.square(lin11), None, None, None, None),
        ((lin11,), (lin11,), np.square(lin11), np.empty(shape=11), None, None, None),
        ((y,), (new_y,), xb + yb, None, (~0,), (~0,), None),
        ((x[..., np.newaxis],), (new_x[..., np.newaxis],), xb + yb, None, (0,), (0,), None),
        ((x[..., np.newaxis],), (0.1 * new_x[..., np.newaxis] + 0.001 * new_y,), x[..., np.newaxis], None,
         (0,), (0,), None),
        ((lin11,), (lin11,), np.square(lin11), None, None, None, 1),
        ((lin11,), (lin11,), np.square(lin11), None, None, None, 0),
    ]
    for k, (ci, co, vi, vo, ai, ao, wi) in enumerate(ml_cases):
        case = f"ml_{k}"
        w = rg.weights(coordinates_input=ci, coordinates_output=co, axis_input=ai, axis_output=ao,
                       weights_input=wi, method="multilinear")
        res = rg.regrid_from_weights(*w, values_input=vi, values_output=None if vo is None else vo.copy(),
                                     axis_input=ai, axis_output=ao)
        store.put_tuple(case, "ci", ci)
        store.put_tuple(case, "co", co)
        store.put(case, "values_input", vi)
        store.put_weights(case, "weights", w)
        store.put(case, "result", res)
        store.set_meta(case, axis_input=None if ai is None else list(ai),
                       axis_output=None if ao is None else list(ao),
                       weights_input=wi, values_output=vo is not None)

    # bounds: _weights_test.py:106-158
    xs = np.array([0.0, 1.0, 2.0, 3.0, 4.0])
    xso = np.array([-0.5, 0.5, 3.5, 4.5])
    case = "bounds"
    store.put(case, "x", xs)
    store.put(case, "x_output", xso)
    store.put(case, "values", xs**2)
    for b in ("extrapolate", "nan"):
        store.put(case, f"result_{b}", rg.regrid(coordinates_input=(xs,), coordinates_output=(xso,),
                                                 values_input=xs**2, method="multilinear", bounds=b))
        store.put_weights(case, f"weights_{b}", rg.weights(coordinates_input=(xs,), coordinates_output=(xso,),
                                                           method="multilinear", bounds=b))

    # conservative 1D: _weights_conservative_1d_test.py:6-152
    c1_cases = [
        (np.linspace(-1, 1, num=11), np.linspace(-1, 1, num=6), np.ones(10), None, None, None),
        (np.linspace(-1, 1, num=11), np.linspace(-1, 1, num=6) + 1e-6, np.ones(10), None, None, None),
        (np.linspace(-1, 1, num=11), np.linspace(-1, 1, num=6) - 1e-6, np.ones(10), None, None, None),
        (np.linspace(1, -1, num=11), np.linspace(-1, 1, num=21), np.ones(10), 0, ~0, None),
        (np.linspace(-1, 1, num=11), np.linspace(1, -1, num=6), np.ones(10), ~0, 0, None),
        (np.linspace(1, -1, num=11), np.linspace(1, -1, num=6), np.ones(10), (0,), 0, None),
        (np.broadcast_to(np.linspace(1, -1, num=11), (3, 4, 11)), np.linspace(1, -1, num=6), np.ones(10), ~0, 0,
         None),
        (np.broadcast_to(np.linspace(1, -1, num=11)[..., np.newaxis, np.newaxis], (11, 3, 4)),
         np.linspace(1, -1, num=6), np.ones(10)[..., np.newaxis, np.newaxis], 0, ~0, None),
        (np.linspace(1, -1, num=11), np.broadcast_to(np.linspace(1, -1, num=6), (3, 4, 6)), np.ones(10), ~0, ~0,
         None),
        (np.linspace(-1, 1, num=11), np.linspace(1, 2, num=6), np.ones(10), None, None, None),
        (np.linspace(1, -1, num=11), np.linspace(1, -1, num=6), np.broadcast_to(np.ones(10), shape=(3, 4, 10)), ~0,
         ~0, None),
        (np.linspace(-1, 1, num=11), np.linspace(-1, 1, num=6), np.ones(10), None, None, 1),
        # non-uniform and reversed grids with a varying weights_input exercise the
        # reversed-index arithmetic of _weights_conservative_1d.py:285-310
        (np.sort(np.random.default_rng(3).uniform(-1, 1, 17))[::-1].copy(),
         np.sort(np.random.default_rng(4).uniform(-1.2, 1.2, 9)), np.arange(1.0, 17.0), None, None,
         np.linspace(0.5, 2.0, 16)),
    ]
    for k, (xi, xo, vi, ai, ao, wi) in enumerate(c1_cases):
        case = f"c1d_{k}"
        w = rg.weights(coordinates_input=xi, coordinates_output=xo, axis_input=ai, axis_output=ao,
                       weights_input=wi, method="conservative")
        res = rg.regrid_from_weights(*w, values_input=vi, axis_input=ai, axis_output=ao)
        store.put(case, "ci", np.ascontiguousarray(xi))
        store.put(case, "co", np.ascontiguousarray(xo))
        store.put(case, "values_input", np.ascontiguousarray(vi))
        if wi is not None:
            store.put(case, "weights_input", wi)
        store.put_weights(case, "weights", w)
        store.put(case, "result", res)

        def ax(a):
            if a is None:
                return None
            return list(a) if isinstance(a, tuple) else int(a)

        store.set_meta(case, axis_input=ax(ai), axis_output=ax(ao), weights_input=wi is not None)

    # find_indices
    fi_cases = [
        ("fi_0", np.linspace(-1, 1, num=32), np.linspace(-1, 1, num=64), None),
        ("fi_1", np.linspace(-1, 1, num=32), np.linspace(-2, 2, num=64), None),
        ("fi_2", np.array([0.0, 1.0, 2.0, 3.0, 4.0]), np.array([-1.0, 0.0, 0.5, 3.5, 4.0, 5.0]), None),
        ("fi_3", np.array([0.0, 1.0, 2.0]), np.array([-1.0, 0.5, 7.0]), -99),
        ("fi_4", np.sort(np.random.default_rng(5).uniform(0, 1, 257)),
         np.random.default_rng(6).uniform(-0.1, 1.1, 300), None),
    ]
    for case, xi, xo, fill in fi_cases:
        store.put(case, "ci", xi)
        store.put(case, "co", xo)
        for method in ("brute", "searchsorted"):
            (res,) = rg.find_indices(coordinates_input=(xi,), coordinates_output=(xo,), method=method,
                                     fill_value=fill)
            store.put(case, f"result_{method}", res)
        store.set_meta(case, fill_value=fill)


# ---------------------------------------------------------------------------
# transposes: _weights_transposed/_weights_transposed_test.py:20-323
# ---------------------------------------------------------------------------


def gen_transposes(store: Store):
    x = np.linspace(-1, 1, num=10)
    y = np.linspace(-1, 1, num=11)
    xb, yb = np.meshgrid(x, y, indexing="ij")
    ci = (xb[..., np.newaxis] + np.array([0, 0.001]), yb[..., np.newaxis] + np.array([0, 0.001]))
    co = (1.1 * (xb[..., np.newaxis] + np.array([0, 0.001])) + 0.01,
          1.2 * (yb[..., np.newaxis] + np.array([0, 0.01])) + 0.001)
    vi = np.random.default_rng(11).normal(size=(x.shape[0] - 1, y.shape[0] - 1, 2))
    w = rg.weights(coordinates_input=ci, coordinates_output=co, axis_input=(0, 1), axis_output=(0, 1),
                   method="conservative")
    data = rg.regrid_from_weights(*w, values_input=vi, axis_input=(0, 1), axis_output=(0, 1))
    wt = rg.transpose_weights(w)
    back = rg.regrid_from_weights(*wt, values_input=data, axis_input=(0, 1), axis_output=(0, 1))
    case = "tw_orth"
    store.put_tuple(case, "ci", ci)
    store.put_tuple(case, "co", co)
    store.put(case, "values_input", vi)
    store.put_weights(case, "weights", w)
    store.put(case, "data", data)
    store.put(case, "back", back)

    x1 = np.linspace(-1, 1, num=10)[..., np.newaxis]
    y1 = np.linspace(-1, 1, num=11)
    x2 = np.linspace(-1, 1, num=5)[..., np.newaxis]
    y2 = np.linspace(-1, 1, num=6)
    twc = [
        (y1, y2, None, None, None),
        (y1, y2, None, None, 2),
        (x1, x2, 0, 0, None),
        ((x1, y1), (x2, y2), None, None, None),
    ]
    for k, (ci, co, ai, ao, wi) in enumerate(twc):
        case = f"twc_{k}"
        w = rg.weights(coordinates_input=ci, coordinates_output=co, axis_input=ai, axis_output=ao,
                       weights_input=wi, method="conservative")
        wtc = rg.transpose_weights_conservative(weights=w, coordinates_input=ci, coordinates_output=co,
                                                axis_input=ai, axis_output=ao, weights_input=wi)
        vals = rg.regrid_from_weights(*wtc, values_input=np.array(10), axis_input=ai, axis_output=ao)
        store.put_tuple(case, "ci", ci)
        store.put_tuple(case, "co", co)
        store.put_weights(case, "weights", w)
        store.put_weights(case, "transposed", wtc)
        store.put(case, "values", vals)
        store.set_meta(case, axis_input=ai, axis_output=ao, weights_input=wi)

    # inverse weighting in 2D: _weights_transposed_test.py:263-323
    rng = np.random.default_rng(0)
    gx = np.linspace(-1, 1, num=8)
    gy = np.linspace(-1, 1, num=12)
    xi, yi = np.meshgrid(gx, gy, indexing="ij")
    xo, yo = xi + 0.03, yi + 0.02
    wi = 1.0 + 0.2 * np.arange(gx.size - 1)[:, None] + 0.05 * np.arange(gy.size - 1)[None, :]
    values = rng.uniform(1, 2, size=(gx.size - 1, gy.size - 1))
    w = rg.weights(coordinates_input=(xi, yi), coordinates_output=(xo, yo), weights_input=wi,
                   method="conservative", perturb=False)
    wtc = rg.transpose_weights_conservative(weights=w, coordinates_input=(xi, yi), coordinates_output=(xo, yo),
                                            weights_input=wi)
    case = "twc_inv2d"
    store.put_tuple(case, "ci", (xi, yi))
    store.put_tuple(case, "co", (xo, yo))
    store.put(case, "weights_input", wi)
    store.put(case, "values", values)
    store.put_weights(case, "weights", w)
    store.put_weights(case, "transposed", wtc)
    store.put(case, "roundtrip", rg.regrid_from_weights(*wtc, values_input=rg.regrid_from_weights(
        *w, values_input=values)))


# ---------------------------------------------------------------------------
# grid helpers: _weights_conservative_2d/_grids_test.py:7-122
# ---------------------------------------------------------------------------


def gen_grids(store: Store):
    for k, (grid, _) in enumerate([
        (np.meshgrid(np.arange(2), np.arange(2), indexing="ij"), None),
        (np.meshgrid(np.arange(3), np.arange(4), indexing="ij"), None),
        (np.meshgrid(2 * np.arange(3), 2 * np.arange(4), indexing="ij"), None),
    ]):
        case = f"area_{k}"
        g = tuple(np.asarray(a, dtype=float) for a in grid)
        store.put_tuple(case, "grid", g)
        store.put(case, "area", _grids.grid_volume(g))
    loc = [
        ((0.5, 0.5), np.meshgrid(np.arange(3), np.arange(4), indexing="ij")),
        ((1.5, 0.5), np.meshgrid(np.arange(3), np.arange(4), indexing="ij")),
        ((1.5, 0.5), np.meshgrid(np.arange(3), np.arange(4))),
        ((-0.5, 2.5), np.meshgrid(-np.arange(3), np.arange(4), indexing="ij")),
        ((-1, -1), np.meshgrid(-np.arange(3), np.arange(4), indexing="ij")),
        ((1, 4.5), np.meshgrid(np.arange(3), np.arange(4), indexing="ij")),
    ]
    for k, (pt, grid) in enumerate(loc):
        case = f"loc_{k}"
        g = tuple(np.asarray(a, dtype=float) for a in grid)
        store.put_tuple(case, "grid", g)
        store.put(case, "point", np.asarray(pt, dtype=float))
        store.put(case, "brute", np.asarray(_grids.index_of_point_brute(pt, g), dtype=np.int64))
        store.put(case, "secant", np.asarray(_grids.index_of_point_secant(pt, g), dtype=np.int64))


# ---------------------------------------------------------------------------
# benchmark-shaped curvilinear grids (cfg1 = the 65^2 -> 49^2 workload)
# ---------------------------------------------------------------------------


def distorted_grid(n: int, angle: float, amp: float, lo: float = -1.0, hi: float = 1.0):
    """Rotate a square ``n x n`` vertex grid, then add ``x += amp sin(pi y)``
    followed by ``y += amp sin(pi x)`` (the second uses the updated x)."""
    a = np.linspace(lo, hi, n)
    x, y = np.meshgrid(a, a, indexing="ij")
    xr = x * np.cos(angle) - y * np.sin(angle)
    yr = x * np.sin(angle) + y * np.cos(angle)
    xr = xr + amp * np.sin(np.pi * yr)
    yr = yr + amp * np.sin(np.pi * xr)
    return xr, yr


def rect_grid(n: int, lo: float, hi: float):
    a = np.linspace(lo, hi, n)
    return tuple(np.meshgrid(a, a, indexing="ij"))


def gen_curvilinear(store: Store):
    # cfg1: 65^2 vertices rotated 0.1, distorted 0.02 -> 49^2 on [-1.1, 1.1]^2,
    # stack of 8 Poisson(100) float64, seed 42, default perturbation
    gi = distorted_grid(65, 0.1, 0.02)
    go = rect_grid(49, -1.1, 1.1)
    values = np.random.default_rng(42).poisson(100, (8, 64, 64)).astype(np.float64)
    case = "cfg1"
    store.put_tuple(case, "ci", gi)
    store.put_tuple(case, "co", go)
    store.put(case, "values_input", values)
    _, cop, *_ = _normalize_input_output_coordinates(gi, go, perturb=True, seed=42)
    store.put_tuple(case, "co_perturbed", cop)
    raw = weights_conservative_2d(gi, tuple(np.ascontiguousarray(c) for c in cop), None)
    store.put(case, "raw_in", raw[0])
    store.put(case, "raw_out", raw[1])
    store.put(case, "raw_val", raw[2])
    w = rg.weights(coordinates_input=gi, coordinates_output=go, method="conservative")
    store.put_weights(case, "weights", w)
    store.put(case, "result", rg.regrid_from_weights(*w, values_input=values))
    store.put(case, "area_input", _grids.grid_volume(gi))

    # other sizes / shapes: 33^2 -> 25^2 (raw + merged), 129^2 -> 97^2 (merged),
    # and the input/output roles swapped with a weights_input
    for n_in, n_out, angle, amp, lo, hi, tag in ((33, 25, 0.3, 0.03, -1.05, 1.05, "curvi33"),
                                                 (129, 97, 0.25, 0.02, -1.05, 1.05, "curvi129")):
        gi = distorted_grid(n_in, angle, amp)
        go = rect_grid(n_out, lo, hi)
        case = tag
        store.put_tuple(case, "ci", gi)
        store.put_tuple(case, "co", go)
        w = rg.weights(coordinates_input=gi, coordinates_output=go, method="conservative")
        store.put_weights(case, "weights", w)
        if n_in <= 33:
            _, cop, *_ = _normalize_input_output_coordinates(gi, go, perturb=True, seed=42)
            raw = weights_conservative_2d(gi, tuple(np.ascontiguousarray(c) for c in cop), None)
            store.put(case, "raw_in", raw[0])
            store.put(case, "raw_out", raw[1])
            store.put(case, "raw_val", raw[2])
            wi = np.linspace(0.5, 2.0, (n_out - 1) ** 2).reshape(n_out - 1, n_out - 1)
            store.put(case, "swap_weights_input", wi)
            store.put_weights(case, "swap_weights", rg.weights(coordinates_input=go, coordinates_output=gi,
                                                               weights_input=wi, method="conservative"))


# ---------------------------------------------------------------------------
# ndarray_linear_interpolation: regridding/_tests/test_interp_ndarray.py:11-93
# (same array sizes and index families; seeded values) plus extrapolated
# indices, orthogonal axes, per-row indices and a reversed axis order
# ---------------------------------------------------------------------------


def gen_interp(store: Store):
    rng = np.random.default_rng(20)
    sz_x, sz_y = 10, 11
    k = 0

    def case(a, indices, axis=None, axis_indices=None):
        nonlocal k
        name = f"interp_{k}"
        k += 1
        store.put(name, "a", a)
        store.put_tuple(name, "indices", tuple(np.asarray(i) for i in indices))
        store.set_meta(name, axis=list(axis) if isinstance(axis, tuple) else axis,
                       axis_indices=list(axis_indices) if isinstance(axis_indices, tuple) else axis_indices)
        store.put(name, "result", rg.ndarray_linear_interpolation(a, indices, axis=axis, axis_indices=axis_indices))

    a1 = rng.random(sz_x)
    for x in (np.arange(sz_x), np.linspace(0, sz_x - 1, num=21)):
        for axis in (None, 0, -1):
            case(a1, (x,), axis)
    a2 = rng.random((sz_x, sz_y))
    for x in (np.arange(sz_x)[:, np.newaxis], np.linspace(0, sz_x - 1, num=100)[:, np.newaxis]):
        for y in (np.arange(sz_y)[np.newaxis, :], np.linspace(0, sz_y - 1, num=5)[np.newaxis, :]):
            xb, yb = np.broadcast_arrays(x, y)
            for axis in (None, (0, 1), (0, ~0)):
                case(a2, (xb, yb), axis)
    # extrapolation (clamped cells), negative and beyond the last sample
    case(a1, (np.linspace(-3.5, sz_x + 2.25, 17),))
    case(a2, tuple(np.broadcast_arrays(np.linspace(-2, sz_x + 1, 7)[:, None], np.linspace(-1.5, sz_y + 3, 9)[None, :])))
    # orthogonal axes: a stack of 2D arrays, indices shared (size-1 axis) or per slice
    a3 = rng.random((9, sz_x, sz_y))
    case(a3, (rng.uniform(0, sz_x - 1, (1, 20)), rng.uniform(0, sz_y - 1, (1, 20))), axis=(1, 2), axis_indices=1)
    case(a3, (rng.uniform(0, sz_x - 1, (9, 20)), rng.uniform(0, sz_y - 1, (9, 20))), axis=(-2, -1), axis_indices=-1)
    # per-row indices along axis 1 of a (9, 10) array, and along axis 0
    a4 = rng.random((9, sz_x))
    case(a4, (rng.uniform(-1, sz_x, (9, 15)),), axis=1, axis_indices=1)
    case(a4, (rng.uniform(0, 8, (1, 15)),), axis=0, axis_indices=1)
    # the interpolation axes given in reverse order
    case(a2, tuple(np.broadcast_arrays(rng.uniform(0, sz_x - 1, (6, 1)), rng.uniform(0, sz_y - 1, (1, 4)))),
         axis=(1, 0))
    # orthogonal broadcasting of a against the indices
    a5 = rng.random((1, sz_x, sz_y))
    case(a5, (rng.uniform(0, sz_x - 1, (3, 7)), rng.uniform(0, sz_y - 1, (3, 7))), axis=(1, 2), axis_indices=1)
    # integer samples
    case(np.arange(12).reshape(3, 4) * 3, (np.array([0.25, 1.5, 2.75]), np.array([0.5, 1.0, 2.5])), axis=(0, 1))


def gen_fill(store: Store):
    """regridding.fill (regridding/_fill/_fill.py:10-109): the inputs of the
    upstream tests (_fill/_fill_test.py:10-119, seeded here), odd and even
    slice sizes with dense missing sets (the periodic neighbours of the
    first/last row and column then share the colour of the cell and the
    sweep order matters), and float64 throughout."""
    rng = np.random.default_rng(30)
    k = 0

    def case(a, where, axis, guess=None, num_iterations=11, **extra):
        nonlocal k
        name = f"fill_{k}"
        k += 1
        store.put(name, "a", a)
        if where is not None:
            store.put(name, "where", where)
        if guess is not None and np.ndim(guess) > 0:
            store.put(name, "guess", guess)
            g_meta = "array"
        else:
            g_meta = guess
        store.set_meta(name, axis=list(axis) if isinstance(axis, tuple) else axis, guess=g_meta,
                       num_iterations=num_iterations, has_where=where is not None, **extra)
        store.put(name, "result", rg.fill(a, where=where, axis=axis, guess=guess, num_iterations=num_iterations))

    nx, ny, nt = 11, 12, 13
    # _fill_test.py:10-49
    for guess in (None, 0.5):
        case(rng.uniform(0, 1, (nx, ny)), rng.uniform(0, 1, (nx, ny)) > 0.9, None, guess)
        case(rng.uniform(0, 1, (nt, nx, ny)), rng.uniform(0, 1, (nt, nx, ny)) > 0.9, (~1, ~0), guess)
        with np.errstate(invalid="ignore"):
            case(np.sqrt(rng.uniform(-0.1, 1, (nx, nt, ny))), None, (0, ~0), guess)
    # _fill_test.py:52-79: zero iterations return the guess
    for guess in (None, 2.0, np.arange(nt, dtype=float).reshape(nt, 1, 1)):
        case(rng.uniform(0, 1, (nt, nx, ny)), rng.uniform(0, 1, (nt, nx, ny)) > 0.9, (~1, ~0), guess, 0)
    # _fill_test.py:82-97: a harmonic field with a missing block
    x = np.linspace(-1, 1, num=32)
    a = x[:, np.newaxis] + 2 * x[np.newaxis, :]
    a[10:16, 10:16] = np.nan
    case(a, None, None, None, 300)
    # _fill_test.py:100-119: a slice with no valid elements
    a = rng.uniform(0, 1, (nt, nx, ny))
    where = rng.uniform(0, 1, a.shape) > 0.9
    where[0] = True
    case(a, where, (~1, ~0), None, 11)
    # odd / even slice sizes, dense missing sets, periodic wrap
    for shape in ((9, 7), (8, 7), (7, 8), (8, 8), (7, 9), (2, 5), (5, 2), (3, 3)):
        for frac in (0.5, 0.95):
            case(rng.uniform(-1, 1, (3,) + shape), rng.uniform(0, 1, (3,) + shape) < frac, (1, 2), None, 7)
    # all cells missing but one, and a guess array varying over the slice
    a = rng.uniform(0, 1, (6, 9))
    where = np.ones(a.shape, dtype=bool)
    where[2, 3] = False
    case(a, where, None, rng.uniform(0, 1, (6, 9)), 5)
    # orthogonal axis in the middle, guess per orthogonal element
    a = rng.uniform(0, 1, (5, 4, 6))
    case(a, rng.uniform(0, 1, a.shape) < 0.4, (0, 2), rng.uniform(0, 1, (1, 4, 1)), 9)
    # where broadcast against a
    a = rng.uniform(0, 1, (4, 7, 8))
    case(a, rng.uniform(0, 1, (7, 8)) < 0.3, (1, 2), None, 6)
    # a 64 x 64 slice pair, 20 iterations (larger sweep)
    a = rng.uniform(0, 1, (2, 64, 64))
    case(a, rng.uniform(0, 1, a.shape) < 0.2, (1, 2), None, 20)


def main(which=None):
    if which is None or "known" in which:
        s = Store()
        gen_conservative_2d(s)
        gen_layout_and_seed(s)
        gen_transposes(s)
        gen_grids(s)
        s.save("known_answers.npz")
    if which is None or "one_dim" in which:
        s = Store()
        gen_1d(s)
        s.save("one_dim.npz")
    if which is None or "curvilinear" in which:
        s = Store()
        gen_curvilinear(s)
        s.save("curvilinear.npz")
    if which is None or "interp" in which:
        s = Store()
        gen_interp(s)
        s.save("interp.npz")
    if which is None or "fill" in which:
        s = Store()
        gen_fill(s)
        s.save("fill.npz")


if __name__ == "__main__":
    # optional arguments: which files to regenerate (known, one_dim, curvilinear, interp, fill)
    main(sys.argv[1:] or None)
