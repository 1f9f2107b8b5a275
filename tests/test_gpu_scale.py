"""Parity at the benchmark sizes, against the oracle on the same inputs.

* 2048^2 -> 1536^2 (quadratic-mapped input, rectilinear output, the default
  perturbation): the built weights equal the oracle's sweep + coalesce
  (the upstream `weights_conservative_2d`, `_weights_conservative_2d.py:76-126`,
  and `_coalesce`, `_weights_arrays.py:44-73`) bit for bit, all 12.8 M
  entries; the exact apply of the benchmark's 64-slice float32 stack equals
  the oracle's float64 apply (`_regrid_from_weights.py:165-182`) bit for
  bit; the compensated apply is within its forward error bound of it (and
  1e-12 relative); the fast float32 apply within the float32 bound; the 2D
  find_indices of a sample of the output vertices equals the oracle's.
* 1024^2 -> 768^2 differentiable workload: weights bit for bit, the values
  gradient against the transposed weights and against
  transpose_weights_conservative, and the adjoint's overlap polygons
  against an accurate float64 overlap (the upstream's own weights are only
  accurate to 1.3e-8 of the cell area at this size; see the test).

The oracle runs on every host core (about 4 s for the 2048^2 build).
"""

import numpy as np
import pytest

import oracle
from overlap import overlap_fraction
from test_gpu_compensated import bound as ff_bound
from test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu

# the adjoint's overlap weights against the accurate overlap at 1024^2
ADJOINT_TOL = 1e-10


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


@pytest.fixture(scope="module")
def cfg2(torch):
    import regridding_gb300 as rg
    from regridding_gb300 import workloads

    gi, go = workloads.cfg2_grids()
    gop = workloads.perturb(go)
    dw = rg.build_conservative_2d(gi, gop)
    exp = oracle.weights_conservative_2d(gi, gop)
    yield gi, gop, dw, exp
    dw.free()


def test_cfg2_weights_bit_exact(cfg2):
    gi, gop, dw, exp = cfg2
    got = dw.export_numpy()
    assert got[2].size == exp[2].size == 12_786_465
    for g, e in zip(got, exp):
        assert_same(g, e)


def test_cfg2_applies(cfg2, torch):
    from regridding_gb300 import workloads

    gi, gop, dw, (ii, oo, vv) = cfg2
    n_out = 1536 * 1536
    d_vals = workloads.cfg2_values_torch(64, 2048, seed=0)
    vals = d_vals.cpu().numpy()
    exp = oracle.apply(ii, oo, vv, vals, n_out)
    # exact: the upstream float64 sums bit for bit
    assert_same(dw.apply(d_vals, accumulate="exact").cpu().numpy(), exp)
    # compensated: forward error bound, and 1e-12 relative on covered cells
    comp = dw.apply(d_vals, accumulate="compensated").cpu().numpy()
    err = np.abs(comp - exp)
    assert np.all(err <= ff_bound(ii, oo, vv, vals, n_out))
    covered = exp != 0
    rel = float(np.max(err[covered] / np.abs(exp[covered])))
    assert rel < 1e-12, rel
    assert np.all(comp[~covered] == 0)
    # fast float32: the float32 FMA chain's bound
    fast = dw.apply(d_vals, accumulate="fast").cpu().numpy()
    k = np.bincount(oo, minlength=n_out)
    b32 = (k + 2) * 2.0**-24 * oracle.apply(ii, oo, np.abs(vv), vals, n_out)
    assert np.all(np.abs(fast - exp) <= b32)


def test_cfg2_find_indices_sample(cfg2):
    """2D find_indices of the output vertices in the 2048^2 input grid: a
    200,000-point sample by the secant method, 64 points (inside and outside)
    by the walk against the exhaustive scan."""
    import regridding_gb300 as rg

    gi, gop, _, _ = cfg2
    rng = np.random.default_rng(8)
    pick = rng.choice(gop[0].size, 200_000, replace=False)
    px, py = gop[0].reshape(-1)[pick], gop[1].reshape(-1)[pick]
    got = rg.locate_2d(gi, px, py, method="secant")
    exp = oracle.locate(gi, px, py, "secant")
    assert_same(got[0], exp[0])
    assert_same(got[1], exp[1])
    assert np.sum(exp[0] == np.iinfo(np.int64).max) > 1000  # outside points among them
    few = pick[:64]
    px, py = gop[0].reshape(-1)[few], gop[1].reshape(-1)[few]
    got = rg.locate_2d(gi, px, py, method="brute")
    exp = oracle.locate(gi, px, py, "brute")
    assert_same(got[0], exp[0])
    assert_same(got[1], exp[1])


def test_cfg4_weights_and_gradients(torch):
    """The 1024^2 -> 768^2 differentiable workload at full size."""
    import regridding_gb300 as rg
    from regridding_gb300 import workloads
    from regridding_gb300.autograd import grad_output_check, regrid_conservative_2d

    gi, go, _ = workloads.cfg4_grids()
    dw = rg.build_conservative_2d(gi, go)
    ii, oo, vv = dw.export_numpy()
    exp = oracle.weights_conservative_2d(gi, go)
    for g, e in zip((ii, oo, vv), exp):
        assert_same(g, e)
    # values gradient = the transposed weights applied to the output gradient
    rng = np.random.default_rng(4)
    v = torch.from_numpy(rng.normal(0, 1, (2, 1024, 1024))).cuda().requires_grad_(True)
    g = rng.normal(0, 1, (2, 768, 768))
    out = regrid_conservative_2d(v, gi, go)
    out.backward(torch.from_numpy(g).cuda())
    got = v.grad.cpu().numpy().reshape(2, -1)
    via_t = oracle.apply(oo, ii, vv, g.reshape(2, -1), 1024 * 1024)
    np.testing.assert_allclose(got, via_t, rtol=1e-13, atol=1e-15)
    # ... and through transpose_weights_conservative (scaled by vol_out / vol_in)
    element = np.empty((), dtype=object)
    element[()] = (ii, oo, vv)
    wt = rg.transpose_weights_conservative((element, (1024, 1024), (768, 768)), gi, go)
    ti, to, tv = wt[0][()]
    vol_in = np.abs(oracle.cell_area_2d(*gi)).ravel()
    vol_out = np.abs(oracle.cell_area_2d(*go)).ravel()
    via_c = oracle.apply(ti, to, tv, g.reshape(2, -1) * vol_out, 1024 * 1024) / vol_in
    np.testing.assert_allclose(got, via_c, rtol=1e-12, atol=1e-14)
    # The adjoint's overlap polygons against an accurate overlap (float64
    # clipping in cell-local coordinates): a 300,000-entry sample and every
    # entry where the adjoint and the upstream weights differ by more than
    # 1e-10.  At this size the upstream's weights themselves (ours are
    # bit-identical) are off from the exact overlap by up to 1.3e-8 of the
    # cell area, where nearly parallel input and output edges make its
    # crossing points ill-conditioned (confirmed in exact rational
    # arithmetic); the adjoint's geometry does not share that error.
    check = grad_output_check(dw, gi, go).cpu().numpy()
    order = np.lexsort((ii, oo))
    ci, co, w = ii[order], oo[order], vv[order]
    far = np.flatnonzero(np.abs(check - w) > 1e-10)
    pick = np.union1d(np.random.default_rng(5).choice(w.size, 300_000, replace=False), far)
    ref = overlap_fraction(gi, go, ci[pick], co[pick])
    err_adjoint = np.abs(check[pick] - ref)
    err_upstream = np.abs(w[pick] - ref)
    assert err_adjoint.max() <= ADJOINT_TOL, (err_adjoint.max(), far.size)
    assert err_upstream.max() <= 2e-8, err_upstream.max()
    assert np.abs(check - w).max() <= 2e-8
    dw.free()
