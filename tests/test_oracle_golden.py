"""Pin the CPU oracle against golden fixtures produced by the upstream package.

Every comparison here is bit-exact: the oracle restates the upstream
pure-Python arithmetic operation for operation.
"""

import numpy as np
import pytest

import fixtures
import oracle

CURVI = fixtures.load("curvilinear.npz")
KNOWN = fixtures.load("known_answers.npz")
ONE = fixtures.load("one_dim.npz")


def perturbed(c):
    """The seed-42 perturbation of the output grid, drawn as the upstream does."""
    rng = np.random.default_rng(42)
    return tuple(rng.normal(a, np.ptp(a, axis=(-1, -2), keepdims=True) * 1e-9) for a in c.tuple("co"))


def assert_same(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape
    assert a.dtype.kind == b.dtype.kind
    assert np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("name", ["cfg1", "curvi33"])
def test_sweep_raw_triples_bit_exact(name):
    c = CURVI.case(name)
    raw = oracle.sweep_2d(c.tuple("ci"), perturbed(c))
    assert_same(raw[0], c["raw_in"])
    assert_same(raw[1], c["raw_out"])
    assert_same(raw[2], c["raw_val"])


def test_perturbation_matches_upstream():
    c = CURVI.case("cfg1")
    for a, b in zip(perturbed(c), c.tuple("co_perturbed")):
        assert_same(a, b)


@pytest.mark.parametrize("name", ["cfg1", "curvi33", "curvi129"])
def test_coalesced_weights_bit_exact(name):
    c = CURVI.case(name)
    got = oracle.weights_conservative_2d(c.tuple("ci"), perturbed(c))
    (exp,) = c.weights()[0].reshape(-1)
    for g, e in zip(got, exp):
        assert_same(g, e)


def test_swapped_roles_with_weights_input():
    c = CURVI.case("curvi33")
    gi, go = c.tuple("ci"), c.tuple("co")
    # the output grid (perturbed) is the second argument of the upstream call
    rng = np.random.default_rng(42)
    gip = tuple(rng.normal(a, np.ptp(a, axis=(-1, -2), keepdims=True) * 1e-9) for a in gi)
    got = oracle.weights_conservative_2d(go, gip, c["swap_weights_input"])
    exp = c.weights("swap_weights")[0][()]
    for g, e in zip(got, exp):
        assert_same(g, e)


def test_cell_area():
    c = CURVI.case("cfg1")
    assert_same(oracle.cell_area_2d(*c.tuple("ci")), c["area_input"])
    for k in range(3):
        a = KNOWN.case(f"area_{k}")
        assert_same(oracle.cell_area_2d(*a.tuple("grid")), a["area"])


@pytest.mark.parametrize("k", range(6))
def test_locate_known_answers(k):
    c = KNOWN.case(f"loc_{k}")
    g = c.tuple("grid")
    p = c["point"]
    for method in ("brute", "secant"):
        oi, oj = oracle.locate(g, p[:1], p[1:], method)
        assert (oi[0], oj[0]) == tuple(c[method])


def test_apply_cfg1_bit_exact():
    c = CURVI.case("cfg1")
    (ii, oo, vv), = c.weights()[0].reshape(-1)
    vin = c["values_input"].reshape(8, -1)
    got = oracle.apply(ii, oo, vv, vin, 48 * 48)
    assert_same(got.reshape(8, 48, 48), c["result"])


@pytest.mark.parametrize("name", ["fi_0", "fi_1", "fi_2", "fi_3", "fi_4"])
def test_find_indices_1d(name):
    c = ONE.case(name)
    for method in ("brute", "searchsorted"):
        got = oracle.find_indices_1d(c["ci"][None], c["co"][None], c.meta["fill_value"], method)[0]
        assert_same(got, c[f"result_{method}"])


def test_multilinear_bounds():
    c = ONE.case("bounds")
    for b in ("extrapolate", "nan"):
        (ii, oo, vv), = oracle.multilinear_1d(c["x"][None], c["x_output"][None], bounds=b)
        got = oracle.coalesce(ii, oo, vv)
        (exp,) = c.weights(f"weights_{b}")[0].reshape(-1)
        for g, e in zip(got, exp):
            assert_same(g, e)
    with pytest.raises(ValueError):
        oracle.multilinear_1d(c["x"][None], c["x_output"][None], bounds="raise")


@pytest.mark.parametrize("k", [0, 1, 2, 9, 11, 12])
def test_conservative_1d(k):
    c = ONE.case(f"c1d_{k}")
    wi = c["weights_input"] if c.has("weights_input") else None
    if wi is not None:
        wi = np.broadcast_to(wi, (c["ci"].size - 1,))
    raw = oracle.conservative_1d(c["ci"], c["co"], wi)
    got = oracle.coalesce(*raw)
    (exp,) = c.weights()[0].reshape(-1)
    for g, e in zip(got, exp):
        assert_same(g, e)


def test_reduceat_model_matches_numpy():
    """The GPU merge sums a group as first + pairwise(rest) with numpy's
    pairwise blocking; this Python model of it must equal add.reduceat."""

    def pw(a):
        n = len(a)
        if n < 8:
            r = -0.0
            for v in a:
                r = r + v
            return r
        if n <= 128:
            r = list(a[:8])
            i = 8
            while i < n - (n % 8):
                for j in range(8):
                    r[j] = r[j] + a[i + j]
                i += 8
            res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]))
            while i < n:
                res = res + a[i]
                i += 1
            return res
        n2 = n // 2
        n2 -= n2 % 8
        return pw(a[:n2]) + pw(a[n2:])

    rng = np.random.default_rng(0)
    for n in list(range(1, 140)) + [300, 1030]:
        a = rng.normal(size=n) * 10.0 ** rng.integers(-3, 17, size=n)
        exp = np.add.reduceat(a, [0])[0]
        got = a[0] + pw(list(a[1:]))
        assert got == exp


def test_degenerate_grids_hit_the_step_cap():
    """Coincident vertices without perturbation: the upstream walk never ends;
    the oracle stops at its step cap and reports an error instead."""
    a = np.linspace(-1, 1, 17)
    x, y = np.meshgrid(a, a, indexing="ij")
    xr, yr = x * np.cos(0.3) - y * np.sin(0.3), x * np.sin(0.3) + y * np.cos(0.3)
    b = np.linspace(-1.05, 1.05, 13)
    xo, yo = np.meshgrid(b, b, indexing="ij")
    with pytest.raises(RuntimeError, match="status 2"):
        oracle.sweep_2d((xr, yr), (xo, yo))


INTERP = fixtures.load("interp.npz")


@pytest.mark.parametrize("k", range(27))
def test_oracle_ndarray_linear_interpolation(k):
    c = INTERP.case(f"interp_{k}")
    meta = c.meta
    axis = tuple(meta["axis"]) if isinstance(meta["axis"], list) else meta["axis"]
    ai = meta["axis_indices"]
    ai = tuple(ai) if isinstance(ai, list) else ai
    got = oracle.ndarray_linear_interpolation(c["a"], c.tuple("indices"), axis=axis, axis_indices=ai)
    np.testing.assert_array_equal(got, c["result"])


FILL = fixtures.load("fill.npz")
N_FILL = 31


def fill_args(k):
    """Inputs of fill fixture k: (a, where, axis, guess, num_iterations)."""
    c = FILL.case(f"fill_{k}")
    meta = c.meta
    axis = tuple(meta["axis"]) if isinstance(meta["axis"], list) else meta["axis"]
    guess = c["guess"] if meta["guess"] == "array" else meta["guess"]
    where = c["where"] if meta["has_where"] else None
    return c["a"], where, axis, guess, meta["num_iterations"], c["result"]


@pytest.mark.parametrize("k", range(N_FILL))
def test_oracle_fill(k):
    a, where, axis, guess, iters, exp = fill_args(k)
    got = oracle.fill(a, where=where, axis=axis, guess=guess, num_iterations=iters)
    assert got.shape == exp.shape
    np.testing.assert_array_equal(got, exp)
