"""Differentiable regrid on the GPU: forward parity with the oracle, the
values gradient against the transposed weights (and its relation to
transpose_weights_conservative), the output-coordinate gradient against
float64 central finite differences (step 1e-7), and the adjoint's overlap
polygons against the built weights."""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def problem(n_in=17, n_out=13, seed=0):
    """Sinusoidally distorted input grid (amplitude 0.02, convex cells) and a
    rectilinear output grid with N(0, 1e-4) vertex jitter."""
    from regridding_gb300 import workloads

    gi = workloads.distorted_grid(n_in, 0.0, 0.02)
    rng = np.random.default_rng(seed)
    go = tuple(c + rng.normal(0, 1e-4, c.shape) for c in workloads.rect_grid(n_out, -0.9, 0.9))
    return gi, go, rng


def test_forward_matches_oracle(torch):
    from regridding_gb300.autograd import regrid_conservative_2d

    gi, go, rng = problem()
    vals = rng.normal(0, 1, (3, 16, 16))
    out = regrid_conservative_2d(torch.from_numpy(vals).cuda(), gi, go).cpu().numpy()
    ii, oo, vv = oracle.weights_conservative_2d(gi, go)
    exp = oracle.apply(ii, oo, vv, vals.reshape(3, -1), 144).reshape(3, 12, 12)
    np.testing.assert_array_equal(out, exp)


def test_values_gradient(torch):
    import regridding_gb300 as rg
    from regridding_gb300.autograd import regrid_conservative_2d

    gi, go, rng = problem(seed=1)
    vals = torch.from_numpy(rng.normal(0, 1, (2, 16, 16))).cuda().requires_grad_(True)
    g = rng.normal(0, 1, (2, 12, 12))
    out = regrid_conservative_2d(vals, gi, go)
    out.backward(torch.from_numpy(g).cuda())
    got = vals.grad.cpu().numpy().reshape(2, -1)
    ii, oo, vv = oracle.weights_conservative_2d(gi, go)
    exp = oracle.apply(oo, ii, vv, g.reshape(2, -1), 256)  # the transposed weights
    np.testing.assert_allclose(got, exp, rtol=1e-13, atol=1e-15)
    # transpose_weights_conservative scales by vol_in / vol_out
    element = np.empty((), dtype=object)
    element[()] = (ii, oo, vv)
    w = (element, (16, 16), (12, 12))
    wt = rg.transpose_weights_conservative(w, gi, go)
    ti, to, tv = wt[0][()]
    vol_in = np.abs(oracle.cell_area_2d(*gi)).ravel()
    vol_out = np.abs(oracle.cell_area_2d(*go)).ravel()
    via = oracle.apply(ti, to, tv, g.reshape(2, -1) * vol_out, 256) / vol_in
    np.testing.assert_allclose(got, via, rtol=1e-12, atol=1e-14)


def test_adjoint_polygons_reproduce_weights(torch):
    import regridding_gb300 as rg
    from regridding_gb300.autograd import grad_output_check

    gi, go, _ = problem(33, 25, seed=2)
    dw = rg.build_conservative_2d(gi, go)
    check = grad_output_check(dw, gi, go).cpu().numpy()
    ii, oo, vv = dw.export_numpy()
    order = np.lexsort((ii, oo))  # CSR order: by output cell, then input cell
    np.testing.assert_allclose(check, vv[order], rtol=0, atol=1e-12)


def coordinate_gradient(torch, dtype, seed=3):
    """Loss 1/2 |regrid(v, grid_in, (x, y)) - target|^2 with the target
    regridded onto the output grid rotated by 0.05 rad; returns the loss
    function, the output grid and the analytic gradients."""
    from regridding_gb300.autograd import regrid_conservative_2d

    gi, go, rng = problem(17, 13, seed=seed)
    vals = rng.normal(0, 1, (4, 16, 16))
    c, s = np.cos(0.05), np.sin(0.05)
    gt = (c * go[0] - s * go[1], s * go[0] + c * go[1])
    v = torch.from_numpy(vals).cuda().to(dtype)
    target = regrid_conservative_2d(v, gi, gt).double().detach()

    def loss(x, y):
        out = regrid_conservative_2d(v, gi, (x, y)).double()
        return 0.5 * ((out - target) ** 2).sum()

    xo = torch.from_numpy(go[0].copy()).cuda().requires_grad_(True)
    yo = torch.from_numpy(go[1].copy()).cuda().requires_grad_(True)
    loss(xo, yo).backward()
    return loss, go, rng, xo.grad.cpu().numpy(), yo.grad.cpu().numpy()


def test_coordinate_gradient_finite_differences(torch):
    """float64: the adjoint against central differences of the forward
    pass (which rebuilds the weights at every shifted coordinate)."""
    loss, go, rng, gx, gy = coordinate_gradient(torch, torch.float64)
    h = 1e-7
    picks = [(int(a), int(b)) for a, b in rng.integers(0, 13, (20, 2))] + [(0, 0), (12, 12), (0, 6), (6, 12)]
    scale = max(np.abs(gx).max(), np.abs(gy).max())
    for which, grad in ((0, gx), (1, gy)):
        for a, b in picks:
            fd = []
            for sgn in (1, -1):
                p = [go[0].copy(), go[1].copy()]
                p[which][a, b] += sgn * h
                with torch.no_grad():
                    fd.append(loss(torch.from_numpy(p[0]).cuda(), torch.from_numpy(p[1]).cuda()).item())
            num = (fd[0] - fd[1]) / (2 * h)
            assert abs(num - grad[a, b]) <= 1e-6 * scale, (which, a, b, num, grad[a, b])


def test_coordinate_gradient_float32_values(torch):
    """float32 values (fast apply): finite differences at this step only see
    float32 rounding, so the float32 gradient is checked against the float64
    one that the previous test pins."""
    _, _, _, gx64, gy64 = coordinate_gradient(torch, torch.float64)
    _, _, _, gx32, gy32 = coordinate_gradient(torch, torch.float32)
    scale = max(np.abs(gx64).max(), np.abs(gy64).max())
    np.testing.assert_allclose(gx32, gx64, rtol=0, atol=1e-4 * scale)
    np.testing.assert_allclose(gy32, gy64, rtol=0, atol=1e-4 * scale)


def test_nonconvex_input_cells_are_refused(torch):
    from regridding_gb300 import _lib
    from regridding_gb300.autograd import regrid_conservative_2d

    a = np.linspace(-1, 1, 9)
    x, y = np.meshgrid(a, a, indexing="ij")
    x = x.copy()
    x[4, 4] += 0.2  # a reflex vertex: cell (4, 4) becomes an arrowhead (positive area, not convex)
    y = y.copy()
    y[4, 4] += 0.2
    go = np.meshgrid(np.linspace(-0.8, 0.8, 6), np.linspace(-0.8, 0.8, 6), indexing="ij")
    xo = torch.from_numpy(go[0]).cuda().requires_grad_(True)
    yo = torch.from_numpy(go[1]).cuda().requires_grad_(True)
    out = regrid_conservative_2d(torch.ones((1, 8, 8), dtype=torch.float64).cuda(), (x, y), (xo, yo))
    with pytest.raises(_lib.RegridError, match="convex"):
        out.sum().backward()


def test_coordinate_gradient_is_deterministic(torch):
    """The coordinate gradient has no atomics: every output vertex sums its
    cells' corner terms in a fixed order, so repeated backward passes give
    the same bits (a 129^2 -> 97^2 case, many cells per vertex row)."""
    from regridding_gb300.autograd import regrid_conservative_2d

    gi, go, rng = problem(129, 97, seed=6)
    v = torch.from_numpy(rng.normal(0, 1, (3, 128, 128))).cuda()
    g = torch.from_numpy(rng.normal(0, 1, (3, 96, 96))).cuda()
    grads = []
    for _ in range(3):
        xo = torch.from_numpy(go[0].copy()).cuda().requires_grad_(True)
        yo = torch.from_numpy(go[1].copy()).cuda().requires_grad_(True)
        regrid_conservative_2d(v, gi, (xo, yo)).backward(g)
        grads.append((xo.grad.cpu().numpy(), yo.grad.cpu().numpy()))
    for gx, gy in grads[1:]:
        np.testing.assert_array_equal(gx, grads[0][0])
        np.testing.assert_array_equal(gy, grads[0][1])
    assert np.abs(grads[0][0]).max() > 0
