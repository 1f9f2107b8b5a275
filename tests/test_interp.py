"""ndarray_linear_interpolation: the host plan (axis normalisation,
broadcasting, flat rows and strides) checked on the CPU by evaluating the
launch it describes with numpy, and the CUDA kernel on the GPU; both
bit-exact against the fixtures produced by the upstream package and against
the oracle on larger random cases."""

import numpy as np
import pytest

import fixtures
import oracle

INTERP = fixtures.load("interp.npz")
N_CASES = 27


def case_args(k):
    c = INTERP.case(f"interp_{k}")
    meta = c.meta
    axis = tuple(meta["axis"]) if isinstance(meta["axis"], list) else meta["axis"]
    ai = meta["axis_indices"]
    ai = tuple(ai) if isinstance(ai, list) else ai
    return c["a"], c.tuple("indices"), axis, ai, c["result"]


def run_plan(p):
    """The rg_interp_linear launch of a plan, evaluated with numpy in the
    kernel's indexing: element e reads row e * stride of each operand."""
    from regridding_gb300 import _interp

    e = np.arange(p.n_orth)[:, None]
    pt = np.arange(p.m)[None, :]
    a = p.rows_a.reshape(-1)
    base_a = e * p.a_stride
    x = p.rows_i[0].reshape(-1)[e * p.i_stride + pt]
    x0 = np.clip(np.floor(x).astype(np.int64), 0, p.nx - 2)
    dx = x - x0
    if p.ny == 0:
        r = a[base_a + x0] * (1 - dx) + a[base_a + x0 + 1] * dx
    else:
        y = p.rows_i[1].reshape(-1)[e * p.i_stride + pt]
        y0 = np.clip(np.floor(y).astype(np.int64), 0, p.ny - 2)
        dy = y - y0
        at = lambda i, j: a[base_a + i * p.ny + j]  # noqa: E731
        r = ((at(x0, y0) * ((1 - dx) * (1 - dy))) + (at(x0, y0 + 1) * ((1 - dx) * dy))
             + (at(x0 + 1, y0) * (dx * (1 - dy))) + (at(x0 + 1, y0 + 1) * (dx * dy)))
    return _interp._finish(p, r)


@pytest.mark.parametrize("k", range(N_CASES))
def test_plan_reproduces_upstream(k):
    from regridding_gb300 import _interp

    a, ind, axis, ai, exp = case_args(k)
    got = run_plan(_interp._plan(a, ind, axis, ai))
    assert got.shape == exp.shape
    np.testing.assert_array_equal(got, exp)


def random_cases():
    rng = np.random.default_rng(5)
    yield rng.normal(0, 1, (6, 40, 30)), (rng.uniform(-2, 41, (6, 500)), rng.uniform(-2, 31, (6, 500))), (1, 2), 1
    yield rng.normal(0, 1, (40, 30, 6)), (rng.uniform(0, 39, (300, 6)), rng.uniform(0, 29, (300, 6))), (0, 1), 0
    yield rng.normal(0, 1, (7, 50)), (rng.uniform(-1, 50, (1, 333)),), 1, 1
    yield rng.normal(0, 1, (1, 64)).astype(np.float32), (rng.uniform(0, 63, (5, 99)),), 1, 1
    yield rng.integers(-9, 9, (33, 17)), (rng.uniform(0, 32, 77), rng.uniform(0, 16, 77)), None, None
    yield rng.normal(0, 1, (4, 3, 20, 21)), (rng.uniform(0, 19, (4, 1, 9, 8)), rng.uniform(0, 20, (1, 3, 9, 8))), \
        (2, 3), (2, 3)


@pytest.mark.parametrize("k", range(6))
def test_plan_random_against_oracle(k):
    from regridding_gb300 import _interp

    a, ind, axis, ai = list(random_cases())[k]
    exp = oracle.ndarray_linear_interpolation(a, ind, axis=axis, axis_indices=ai)
    got = run_plan(_interp._plan(a, ind, axis, ai))
    np.testing.assert_array_equal(got, exp)


def test_plan_errors():
    from regridding_gb300 import _interp

    a = np.zeros((4, 5))
    with pytest.raises(ValueError, match="number of indices"):
        _interp._plan(a, (np.zeros(3),), None, None)
    with pytest.raises(ValueError, match="at least 2 samples"):
        _interp._plan(np.zeros((1, 5)), (np.zeros(3), np.zeros(3)), None, None)
    with pytest.raises(ValueError, match="orthogonal"):
        _interp._plan(np.zeros((3, 4, 5)), (np.zeros(7), np.zeros(7)), (1, 2), 0)
    p = _interp._plan(a, (np.zeros((0,)), np.zeros((0,))), None, None)
    assert p.m == 0


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(N_CASES))
def test_gpu_reproduces_upstream(torch, k):
    import regridding_gb300 as rg

    a, ind, axis, ai, exp = case_args(k)
    got = rg.ndarray_linear_interpolation(a, ind, axis=axis, axis_indices=ai)
    assert got.shape == exp.shape and got.dtype == np.float64
    np.testing.assert_array_equal(got, exp)


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(6))
def test_gpu_random_against_oracle(torch, k):
    import regridding_gb300 as rg

    a, ind, axis, ai = list(random_cases())[k]
    exp = oracle.ndarray_linear_interpolation(a, ind, axis=axis, axis_indices=ai)
    np.testing.assert_array_equal(rg.ndarray_linear_interpolation(a, ind, axis=axis, axis_indices=ai), exp)


@pytest.mark.gpu
def test_gpu_nonfinite_and_huge_indices(torch):
    """NaN indices give NaN; infinite and huge indices land in the first or
    last cell (the conversion saturates and the cell is clamped)."""
    import regridding_gb300 as rg

    a = np.arange(10.0) ** 2
    x = np.array([np.nan, 1e300, -1e300, np.inf, -np.inf, 2.5, 9.0, 0.0])
    got = rg.ndarray_linear_interpolation(a, (x,))
    assert np.isnan(got[0])
    with np.errstate(invalid="ignore"):
        exp = oracle.ndarray_linear_interpolation(a, (x[5:],))
    np.testing.assert_array_equal(got[5:], exp)
    # x = +-1e300 extrapolates the last / first cell: huge, of the right sign
    assert got[1] > 1e300 and got[2] < -1e299


@pytest.mark.gpu
def test_gpu_large_stack(torch):
    """A (64, 512, 512) stack at 4096 points per slice, against the oracle."""
    import regridding_gb300 as rg

    rng = np.random.default_rng(9)
    a = rng.normal(0, 1, (64, 512, 512))
    x = rng.uniform(-3, 514, (64, 4096))
    y = rng.uniform(-3, 514, (64, 4096))
    got = rg.ndarray_linear_interpolation(a, (x, y), axis=(1, 2), axis_indices=1)
    np.testing.assert_array_equal(got, oracle.ndarray_linear_interpolation(a, (x, y), axis=(1, 2), axis_indices=1))
