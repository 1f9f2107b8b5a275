"""The compensated apply (``accumulate="compensated"``, RG_ACC_COMPENSATED):
float32 stacks, float64 output, float-float arithmetic on the FP32 pipe.

Tolerance: the result is checked against the oracle's float64 apply (the
upstream loop, `_regrid_from_weights.py:165-182`) with the forward error
bound of the method plus that of the oracle's own float64 sum,

    |got - oracle| <= (1.5 * 2^-47 + (n + 2)^2 * 2^-48 + (n + 2) * 2^-53) * sum_k |w_k x_k|,

n the row's entry count; with positive data that is a relative bound, and
rows up to 14 entries are within 1e-12.  Outputs whose float32 partial sum
overflows, and rows that read a non-finite input, are recomputed in float64
in the upstream order, so they equal the oracle bit for bit.
"""

import ctypes

import numpy as np
import pytest

import oracle
from test_gpu_parity import _local_coo, assert_same

pytestmark = pytest.mark.gpu

# the compensated kernel's configurations (slices per stage, stages, register
# cap, entries held in registers), as RG_APPLY_FF_CONFIG forces them
FF_CONFIGS = ["6,2,0,6", "8,2,0,6", "4,2,0,6", "4,3,0,6", "2,4,0,6", "4,3,3,4", "4,2,4,0"]


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def bound(ii, oo, vv, vals, n_out):
    k = np.bincount(oo, minlength=n_out).astype(np.float64)
    s = oracle.apply(ii, oo, np.abs(vv), np.abs(vals).astype(np.float64), n_out)
    return (1.5 * 2.0**-47 + (k + 2) ** 2 * 2.0**-48 + (k + 2) * 2.0**-53) * s


def check_handle(dw, torch):
    from regridding_gb300 import _lib

    _lib.call("rg_weights_check", dw.handle, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def make(case, rng, torch):
    from regridding_gb300 import _lib
    from regridding_gb300._device import DeviceWeights

    n0_in, n1_in, n0_out, n1_out = 40, 48, 30, 37
    kw = {}
    if case == "long_lists":
        kw = {"spread": 6}
    if case == "tma_all_far":
        kw = {"spread": 3}
    if case == "long_rows":
        kw = {"per_row": (12, 30)}
    ii, oo, vv = _local_coo(rng, n0_in, n1_in, n0_out, n1_out, **kw)
    n_in = n0_in * n1_in
    n_out = n0_out * n1_out
    if case == "tma_some_far":
        key = np.unique(np.concatenate([oo * n_in + ii, np.array([5, 200, 611, 1000]) * n_in + [1913, 3, 960, 47]]))
        oo, ii = key // n_in, key % n_in
        vv = rng.uniform(0.1, 1.0, ii.size)
    if case == "long_rows":
        # rows of 12-30 entries (a 5x5 neighbourhood read by every output)
        ii, oo = [], []
        for o in range(n_out):
            i, j = divmod(o, n1_out)
            ci, cj = int(i * n0_in / n0_out), int(j * n1_in / n1_out)
            cells = np.unique(np.clip(ci + rng.integers(-2, 3, 30), 0, n0_in - 1) * n1_in +
                              np.clip(cj + rng.integers(-2, 3, 30), 0, n1_in - 1))
            ii.extend(cells.tolist())
            oo.extend([o] * len(cells))
        ii, oo = np.asarray(ii, np.int64), np.asarray(oo, np.int64)
        vv = rng.uniform(0.01, 1.0, ii.size)
    shape = None if case == "no_shape" else (n0_out, n1_out)
    dw = DeviceWeights.from_coo(ii, oo, vv, n_in, n_out, shape)
    if case != "no_shape":
        _lib.call("rg_weights_set_input_shape", dw.handle, n0_in, n1_in)
    return dw, ii, oo, vv, n_in, n_out


@pytest.mark.parametrize("case", ["tma", "tma_some_far", "tma_all_far", "long_lists", "long_rows", "no_shape",
                                  "unaligned"])
@pytest.mark.parametrize("stack", [1, 3, 7, 64])
def test_compensated_paths(torch, case, stack):
    """Every path the compensated mode takes (tensor-copy staging for all
    patches, for all but a few, or none; no shapes or an unaligned stack,
    which compute as the exact apply) is within the bound of the oracle, and
    applying again gives the same bits."""
    rng = np.random.default_rng([7, len(case), sum(map(ord, case)), stack])
    dw, ii, oo, vv, n_in, n_out = make(case, rng, torch)
    vals = rng.lognormal(0, 2, (stack, n_in)).astype(np.float32)
    if case == "unaligned":
        buf = torch.empty(stack * n_in + 1, dtype=torch.float32, device="cuda")
        d_vals = buf[1:].view(stack, n_in)
        d_vals.copy_(torch.from_numpy(vals))
    else:
        d_vals = torch.from_numpy(vals).cuda()
    got = dw.apply(d_vals, accumulate="compensated").cpu().numpy()
    assert got.dtype == np.float64 and got.shape == (stack, n_out)
    exp = oracle.apply(ii, oo, vv, vals, n_out)
    b = bound(ii, oo, vv, vals, n_out)
    err = np.abs(got - exp)
    assert np.all(err <= b), float(np.max(err / np.maximum(b, 1e-300)))
    if case in ("no_shape", "unaligned"):
        assert_same(got, exp)  # computed by the exact apply
    # positive data: the relative error is far inside 1e-12
    rel = err / np.maximum(np.abs(exp), 1e-300)
    assert float(rel.max()) < (1e-12 if case != "long_rows" else 5e-12)
    again = dw.apply(d_vals, accumulate="compensated").cpu().numpy()
    assert_same(again, got)
    check_handle(dw, torch)


def test_compensated_on_built_weights(torch):
    """Conservative weights of a distorted 257^2 -> 193^2 pair, a log-normal
    float32 stack: within 1e-12 relative of the upstream float64 apply
    (measured ~1e-15); the fast and exact modes on the same handle keep
    their own results."""
    import regridding_gb300 as rg
    from regridding_gb300 import workloads

    gi = workloads.distorted_grid(257, 0.25, 0.02)
    go = workloads.perturb(workloads.rect_grid(193, -1.05, 1.05))
    dw = rg.build_conservative_2d(gi, go)
    ii, oo, vv = dw.export_numpy()
    rng = np.random.default_rng(3)
    vals = rng.lognormal(3, 1, (16, 256 * 256)).astype(np.float32)
    d_vals = torch.from_numpy(vals).cuda()
    exact = dw.apply(d_vals, accumulate="exact").cpu().numpy()
    comp = dw.apply(d_vals, accumulate="compensated").cpu().numpy()
    fast = dw.apply(d_vals, accumulate="fast").cpu().numpy()
    exp = oracle.apply(ii, oo, vv, vals, 192 * 192)
    assert_same(exact, exp)
    assert np.all(np.abs(comp - exp) <= bound(ii, oo, vv, vals, 192 * 192))
    covered = np.abs(exp) > 0
    assert float(np.max(np.abs(comp - exp)[covered] / np.abs(exp[covered]))) < 1e-12
    assert np.all(comp[~covered] == 0)
    np.testing.assert_allclose(fast, exp, rtol=1e-6, atol=1e-6 * exp.max())
    assert_same(dw.apply(d_vals, accumulate="exact").cpu().numpy(), exact)
    check_handle(dw, torch)


@pytest.mark.parametrize("stack", [1, 7, 64])
def test_compensated_box_configs_agree(torch, stack, monkeypatch):
    """Every configuration of the tensor-copy kernel computes each output's
    float-float chain in the same order: identical bits whichever is forced."""
    from regridding_gb300 import _lib
    from regridding_gb300._device import DeviceWeights

    rng = np.random.default_rng([101, stack])
    n0_in, n1_in, n0_out, n1_out = 64, 96, 48, 60
    ii, oo, vv = _local_coo(rng, n0_in, n1_in, n0_out, n1_out)
    n_in, n_out = n0_in * n1_in, n0_out * n1_out
    vals = rng.lognormal(1, 1, (stack, n_in)).astype(np.float32)
    d_vals = torch.from_numpy(vals).cuda()
    results = []
    for cfg in FF_CONFIGS:
        monkeypatch.setenv("RG_APPLY_FF_CONFIG", cfg)
        dw = DeviceWeights.from_coo(ii, oo, vv, n_in, n_out, (n0_out, n1_out))
        _lib.call("rg_weights_set_input_shape", dw.handle, n0_in, n1_in)
        results.append(dw.apply(d_vals, accumulate="compensated").cpu().numpy())
        dw.free()
    for cfg, got in zip(FF_CONFIGS[1:], results[1:]):
        np.testing.assert_array_equal(got, results[0], err_msg=cfg)
    exp = oracle.apply(ii, oo, vv, vals, n_out)
    assert np.all(np.abs(results[0] - exp) <= bound(ii, oo, vv, vals, n_out))


def test_compensated_non_finite_and_overflow(torch):
    """Inputs near the float32 maximum whose float32 partial sums overflow,
    infinities, NaNs, negative values and weights: such outputs are
    recomputed in float64 in the upstream order (bit-identical to the
    oracle, NaN where the upstream gives NaN); the rest stay within the
    bound."""
    rng = np.random.default_rng(17)
    dw, ii, oo, vv, n_in, n_out = make("tma", rng, torch)
    vals = rng.normal(0, 1, (8, n_in)).astype(np.float32)
    vals[0, ::7] = 3.0e38
    vals[1, 5] = np.inf
    vals[2, 9] = -np.inf
    vals[3, 11] = np.nan
    vals[4, :] = 3.3e38
    d_vals = torch.from_numpy(vals).cuda()
    got = dw.apply(d_vals, accumulate="compensated").cpu().numpy()
    with np.errstate(all="ignore"):
        exp = oracle.apply(ii, oo, vv, vals, n_out)
        b = bound(ii, oo, vv, vals, n_out)
    finite = np.isfinite(exp) & np.isfinite(b)
    special = ~finite | (np.abs(exp) > 1e38)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(exp))
    np.testing.assert_array_equal(got[~finite], exp[~finite])
    big = finite & (np.abs(exp) > 1e38)
    assert big.any()
    assert np.all(np.abs(got[big] - exp[big]) <= b[big])
    ok = finite & ~special
    assert np.all(np.abs(got[ok] - exp[ok]) <= b[ok])
    check_handle(dw, torch)


def test_compensated_from_host_buffers(torch):
    """rg_apply_host with RG_ACC_COMPENSATED (chunks of slices copied in,
    applied and copied out on separate streams) equals the device apply."""
    from regridding_gb300 import _lib

    rng = np.random.default_rng(23)
    dw, ii, oo, vv, n_in, n_out = make("tma", rng, torch)
    vals = rng.lognormal(2, 1, (37, n_in)).astype(np.float32)
    dev = dw.apply(torch.from_numpy(vals).cuda(), accumulate="compensated").cpu().numpy()
    h_in = torch.from_numpy(vals).pin_memory()
    h_out = torch.empty((37, n_out), dtype=torch.float64).pin_memory()
    s = torch.cuda.current_stream()
    _lib.call("rg_apply_host", dw.handle, ctypes.c_void_p(h_in.data_ptr()), _lib.RG_F32,
              ctypes.c_void_p(h_out.data_ptr()), _lib.RG_F64, 37, _lib.RG_ACC_COMPENSATED, 5,
              ctypes.c_void_p(s.cuda_stream))
    s.synchronize()
    assert_same(h_out.numpy(), dev)


def test_compensated_public_api(torch):
    """regrid_from_weights(..., accumulate="compensated") returns float64
    within the bound; float64 input computes as the exact apply."""
    import regridding_gb300 as rg
    from regridding_gb300 import workloads

    gi, go, values = workloads.cfg1()
    w = rg.weights(gi, go, method="conservative")
    v32 = values.astype(np.float32)
    got = rg.regrid_from_weights(*w, values_input=v32, accumulate="compensated")
    exact = rg.regrid_from_weights(*w, values_input=v32)
    assert got.dtype == np.float64
    np.testing.assert_allclose(got, exact, rtol=1e-12, atol=0)
    assert_same(rg.regrid_from_weights(*w, values_input=values, accumulate="compensated"),
                rg.regrid_from_weights(*w, values_input=values))
    with pytest.raises(ValueError):
        rg.regrid_from_weights(*w, values_input=values, accumulate="double")
