"""fill(method="gauss_seidel"): the host plan (broadcasting, axes, moved
layout, guess kinds) checked on the CPU by running the oracle's sweep on the
plan's arrays, and the CUDA path on the GPU; bit-exact against the fixtures
produced by the upstream package (float64) and against the oracle on larger
cases (float64 and float32)."""

import numpy as np
import pytest

import fixtures
import oracle

FILL = fixtures.load("fill.npz")
N_FILL = 31


def fill_args(k):
    c = FILL.case(f"fill_{k}")
    meta = c.meta
    axis = tuple(meta["axis"]) if isinstance(meta["axis"], list) else meta["axis"]
    guess = c["guess"] if meta["guess"] == "array" else meta["guess"]
    where = c["where"] if meta["has_where"] else None
    return c["a"], where, axis, guess, meta["num_iterations"], c["result"]


def run_plan(a, where, axis, guess, iters):
    """The launch described by the host plan, evaluated by the oracle: seed
    (median / per-slice / per-cell guess), then the sequential sweep."""
    from regridding_gb300 import _fill, _lib

    if where is None:
        where = np.isnan(a)
    rows, mask, kind, g, axis_n, moved_shape = _fill._plan(a, where, axis, guess)
    rows = rows.copy()
    m = mask.astype(bool)
    if kind == _lib.RG_FILL_GUESS_MEDIAN:
        g = oracle.fill_median_guess(rows, m, (1, 2))
    elif kind == _lib.RG_FILL_GUESS_SLICE:
        g = g[:, None, None]
    rows[m] = np.broadcast_to(g, rows.shape)[m]
    out = oracle.fill(rows, where=m, axis=(1, 2), guess=rows, num_iterations=iters)
    return np.moveaxis(out.reshape(moved_shape), (-2, -1), axis_n)


@pytest.mark.parametrize("k", range(N_FILL))
def test_plan_reproduces_upstream(k):
    a, where, axis, guess, iters, exp = fill_args(k)
    got = run_plan(a, where, axis, guess, iters)
    assert got.shape == exp.shape
    np.testing.assert_array_equal(got, exp)


def test_plan_errors():
    from regridding_gb300 import _fill

    with pytest.raises(ValueError, match="interpolation axes"):
        _fill._plan(np.zeros((3, 4, 5)), np.zeros((3, 4, 5), bool), None, None)
    with pytest.raises(ValueError, match="Unrecognized method"):
        import regridding_gb300 as rg

        rg.fill(np.zeros((3, 4)), method="sor")


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(N_FILL))
def test_gpu_reproduces_upstream(torch, k):
    import regridding_gb300 as rg

    a, where, axis, guess, iters, exp = fill_args(k)
    got = rg.fill(a, where=where, axis=axis, guess=guess, num_iterations=iters)
    assert got.shape == exp.shape and got.dtype == exp.dtype
    np.testing.assert_array_equal(got, exp)


def large_cases():
    rng = np.random.default_rng(31)
    # blocks of missing cells on 4 slices of 301 x 257 (odd x odd), 40 iterations
    a = rng.normal(0, 1, (4, 301, 257))
    where = np.zeros(a.shape, bool)
    for _ in range(60):
        t, j, i = rng.integers(0, 4), rng.integers(0, 290), rng.integers(0, 250)
        where[t, j:j + rng.integers(2, 12), i:i + rng.integers(2, 8)] = True
    yield a, where, (1, 2), None, 40
    # 30 % random missing, even x odd, the slice axis last, per-cell guess
    a = rng.normal(0, 1, (128, 95, 3))
    yield a, rng.uniform(0, 1, a.shape) < 0.3, (0, 1), rng.normal(0, 1, a.shape), 25
    # dense missing set on an odd x even float32 stack
    a = rng.normal(0, 1, (6, 63, 64)).astype(np.float32)
    yield a, rng.uniform(0, 1, a.shape) < 0.9, (1, 2), None, 30
    # NaNs at the valid cells too (they propagate) and an all-missing slice
    a = rng.normal(0, 1, (3, 40, 41))
    a[1, 5, 5] = np.nan
    where = rng.uniform(0, 1, a.shape) < 0.2
    where[2] = True
    yield a, where, (1, 2), None, 15


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(4))
def test_gpu_against_oracle(torch, k):
    import regridding_gb300 as rg

    a, where, axis, guess, iters = list(large_cases())[k]
    exp = oracle.fill(a, where=where, axis=axis, guess=guess, num_iterations=iters)
    got = rg.fill(a, where=where, axis=axis, guess=guess, num_iterations=iters)
    assert got.dtype == exp.dtype
    np.testing.assert_array_equal(got, exp)


@pytest.mark.gpu
def test_gpu_median(torch):
    """rg_fill_median against numpy's nanmedian: odd and even counts, ties,
    NaNs among the valid cells, negative values and an empty slice."""
    from regridding_gb300 import _device, _lib

    rng = np.random.default_rng(32)
    for dtype, code in ((np.float64, _lib.RG_F64), (np.float32, _lib.RG_F32)):
        a = rng.normal(0, 1, (7, 1001)).astype(dtype)
        a[2] = np.round(a[2])  # many ties
        a[3, ::7] = np.nan
        where = rng.uniform(0, 1, a.shape) < 0.3
        where[4] = True
        where[5, 1:] = True  # one valid element
        where[6, 2:] = True  # two
        exp = oracle.fill_median_guess(a, where, (1,))[:, 0]
        out = torch.empty(7, dtype=torch.float64 if dtype == np.float64 else torch.float32, device="cuda")
        d_a = _device.upload(a)
        d_w = _device.upload(where.astype(np.uint8))
        _lib.call("rg_fill_median", _device.ptr(d_a), code, _device.ptr(d_w), 7, 1001, _device.ptr(out),
                  _device.stream())
        np.testing.assert_array_equal(out.cpu().numpy(), exp.astype(dtype))


@pytest.mark.gpu
def test_gpu_axis_of_length_one(torch):
    import regridding_gb300 as rg

    a = np.ones((5, 1))
    a[2, 0] = np.nan
    with pytest.raises(ZeroDivisionError):
        rg.fill(a)
    np.testing.assert_array_equal(rg.fill(a, num_iterations=0), np.ones((5, 1)))
