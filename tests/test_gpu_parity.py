"""GPU parity: the CUDA path against the upstream's own outputs (golden
fixtures) and against the CPU oracle at sizes the fixtures do not reach.

Tolerances: indices and weights are compared bit for bit (the kernels follow
the upstream arithmetic exactly); exact-mode applies are bit for bit; the
float32 fast apply is checked to 1e-6 relative.
"""

import ctypes

import numpy as np
import pytest

import fixtures
import oracle

pytestmark = pytest.mark.gpu

KNOWN = fixtures.load("known_answers.npz")
ONE = fixtures.load("one_dim.npz")
CURVI = fixtures.load("curvilinear.npz")


@pytest.fixture(scope="module")
def rg():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import regridding_gb300

    return regridding_gb300


def assert_same(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    assert np.array_equal(a, b, equal_nan=True), np.max(np.abs(a - b)) if a.dtype.kind == "f" else None


def assert_weights_same(got, exp):
    ga, gs_in, gs_out = got
    ea, es_in, es_out = exp
    assert tuple(gs_in) == tuple(es_in) and tuple(gs_out) == tuple(es_out)
    assert ga.shape == ea.shape
    for g, e in zip(ga.reshape(-1), ea.reshape(-1)):
        for x, y in zip(g, e):
            assert_same(x, y)


def kw_axes(meta):
    out = {}
    for k in ("axis_input", "axis_output"):
        v = meta.get(k)
        out[k] = tuple(v) if isinstance(v, list) else v
    return out


# ---------------------------------------------------------------------------
# conservative 2D known answers
# ---------------------------------------------------------------------------


@pytest.mark.parametrize("k", range(15))
def test_conservative_2d_known_answers(rg, k):
    c = KNOWN.case(f"c2d_{k}")
    wi = c["weights_input"] if c.has("weights_input") else None
    w = rg.weights(c.tuple("ci"), c.tuple("co"), weights_input=wi, method="conservative", perturb=False)
    assert_weights_same(w, c.weights())
    res = rg.regrid_from_weights(*w, values_input=c["values_input"])
    assert_same(res, c["result"])
    assert np.allclose(res, c["expected"], rtol=1e-3)


def test_saved_layout_contract(rg):
    c = KNOWN.case("layout")
    ci, co = c.tuple("ci"), c.tuple("co")
    w = rg.weights(ci, co, method="conservative")
    assert_weights_same(w, c.weights())
    for ii, oo, vv in w[0].reshape(-1):
        assert ii.dtype == np.int64 and oo.dtype == np.int64 and vv.dtype == np.float64
        key = ii * (oo.max() + 1) + oo
        assert np.unique(key).size == key.size
    vals = c["values_input"]
    assert_same(rg.regrid_from_weights(*w, values_input=vals), c["result"])
    assert_same(rg.regrid(ci, co, values_input=vals, method="conservative"), c["result"])
    assert_same(rg.regrid(ci, co, values_input=vals, method="conservative"), c["regrid"])
    # pickle round trip gives a bit-identical apply
    import pickle

    w2 = pickle.loads(pickle.dumps(w))
    assert_same(rg.regrid_from_weights(*w2, values_input=vals), c["result"])
    # transposes
    wt = rg.transpose_weights(w)
    assert wt[1] == w[2] and wt[2] == w[1]
    for t_el, el in zip(wt[0].reshape(-1), w[0].reshape(-1)):
        assert t_el[0] is el[1] and t_el[1] is el[0] and t_el[2] is el[2]
    wtc = rg.transpose_weights_conservative(w, ci, co)
    assert_weights_same(wtc, c.weights("transposed_conservative"))
    back = rg.regrid_from_weights(*wtc, values_input=rg.regrid_from_weights(*w, values_input=vals))
    assert_same(back, c["roundtrip"])


@pytest.mark.parametrize("tag", ["default", "s12345", "s0", "s1", "gen12345", "unperturbed"])
def test_seeded_perturbation(rg, tag):
    c = KNOWN.case("seed")
    kw = {"default": {}, "s12345": {"seed": 12345}, "s0": {"seed": 0}, "s1": {"seed": 1},
          "gen12345": {"seed": np.random.default_rng(12345)}, "unperturbed": {"perturb": False}}[tag]
    w = rg.weights(c.tuple("ci"), c.tuple("co"), method="conservative", **kw)
    assert_weights_same(w, c.weights(f"w_{tag}"))


def test_transpose_orthogonal_axis(rg):
    c = KNOWN.case("tw_orth")
    ci, co = c.tuple("ci"), c.tuple("co")
    w = rg.weights(ci, co, axis_input=(0, 1), axis_output=(0, 1), method="conservative")
    assert_weights_same(w, c.weights())
    data = rg.regrid_from_weights(*w, values_input=c["values_input"], axis_input=(0, 1), axis_output=(0, 1))
    assert_same(data, c["data"])
    back = rg.regrid_from_weights(*rg.transpose_weights(w), values_input=data, axis_input=(0, 1),
                                  axis_output=(0, 1))
    assert_same(back, c["back"])


@pytest.mark.parametrize("k", range(4))
def test_transpose_conservative(rg, k):
    c = KNOWN.case(f"twc_{k}")
    ci, co = c.tuple("ci"), c.tuple("co")
    ai, ao, wi = c.meta["axis_input"], c.meta["axis_output"], c.meta["weights_input"]
    if len(ci) == 1:
        ci, co = ci[0], co[0]
    w = rg.weights(ci, co, axis_input=ai, axis_output=ao, weights_input=wi, method="conservative")
    assert_weights_same(w, c.weights())
    wtc = rg.transpose_weights_conservative(w, ci, co, axis_input=ai, axis_output=ao, weights_input=wi)
    assert_weights_same(wtc, c.weights("transposed"))
    vals = rg.regrid_from_weights(*wtc, values_input=np.array(10), axis_input=ai, axis_output=ao)
    assert_same(vals, c["values"])


def test_transpose_conservative_inverts_weights_input_2d(rg):
    c = KNOWN.case("twc_inv2d")
    ci, co, wi = c.tuple("ci"), c.tuple("co"), c["weights_input"]
    w = rg.weights(ci, co, weights_input=wi, method="conservative", perturb=False)
    assert_weights_same(w, c.weights())
    wtc = rg.transpose_weights_conservative(w, ci, co, weights_input=wi)
    assert_weights_same(wtc, c.weights("transposed"))
    rt = rg.regrid_from_weights(*wtc, values_input=rg.regrid_from_weights(*w, values_input=c["values"]))
    assert_same(rt, c["roundtrip"])


# ---------------------------------------------------------------------------
# 1D
# ---------------------------------------------------------------------------


@pytest.mark.parametrize("k", range(7))
def test_multilinear_known_answers(rg, k):
    c = ONE.case(f"ml_{k}")
    kw = kw_axes(c.meta)
    ci, co = c.tuple("ci"), c.tuple("co")
    w = rg.weights(ci, co, weights_input=c.meta["weights_input"], method="multilinear", **kw)
    assert_weights_same(w, c.weights())
    vo = np.empty(shape=11) if c.meta["values_output"] else None
    res = rg.regrid_from_weights(*w, values_input=c["values_input"], values_output=vo, **kw)
    assert res.dtype == np.float64
    assert_same(res, c["result"])


def test_multilinear_bounds(rg):
    c = ONE.case("bounds")
    x, xo = c["x"], c["x_output"]
    for b in ("extrapolate", "nan"):
        w = rg.weights((x,), (xo,), method="multilinear", bounds=b)
        assert_weights_same(w, c.weights(f"weights_{b}"))
        res = rg.regrid((x,), (xo,), values_input=c["values"], method="multilinear", bounds=b)
        assert_same(res, c[f"result_{b}"])
    with pytest.raises(ValueError, match="fall outside the input grid"):
        rg.regrid((x,), (xo,), values_input=c["values"], method="multilinear", bounds="raise")
    inside = rg.regrid((x,), (np.array([0.5, 3.5]),), values_input=c["values"], method="multilinear",
                       bounds="raise")
    assert np.allclose(inside, [0.5, 12.5])
    with pytest.raises(ValueError, match="Unrecognized bounds="):
        rg.regrid((x,), (xo,), values_input=c["values"], method="multilinear", bounds="foo")


@pytest.mark.parametrize("k", range(13))
def test_conservative_1d_known_answers(rg, k):
    c = ONE.case(f"c1d_{k}")
    ai, ao = c.meta["axis_input"], c.meta["axis_output"]
    ai = tuple(ai) if isinstance(ai, list) else ai
    ao = tuple(ao) if isinstance(ao, list) else ao
    wi = c["weights_input"] if c.has("weights_input") else None
    w = rg.weights(c["ci"], c["co"], axis_input=ai, axis_output=ao, weights_input=wi, method="conservative")
    assert_weights_same(w, c.weights())
    res = rg.regrid_from_weights(*w, values_input=c["values_input"], axis_input=ai, axis_output=ao)
    assert_same(res, c["result"])


@pytest.mark.parametrize("name", ["fi_0", "fi_1", "fi_2", "fi_3", "fi_4"])
def test_find_indices_1d(rg, name):
    c = ONE.case(name)
    for method in ("brute", "searchsorted"):
        (got,) = rg.find_indices((c["ci"],), (c["co"],), method=method, fill_value=c.meta["fill_value"])
        assert_same(got, c[f"result_{method}"])
    with pytest.raises(ValueError):
        rg.find_indices((c["ci"],), (c["co"],), method="invalid method")


def test_find_indices_1d_batched_against_oracle(rg):
    rng = np.random.default_rng(7)
    xi = np.sort(rng.uniform(0, 1, (40, 300)), axis=-1)
    xi[3] = xi[3][::-1]  # a descending row: brute scans it linearly
    xo = rng.uniform(-0.05, 1.05, (40, 500))
    xo[5, :7] = xi[5, :7]  # points exactly on vertices
    for method in ("brute", "searchsorted"):
        (got,) = rg.find_indices((xi,), (xo,), axis_input=-1, axis_output=-1, method=method)
        exp = oracle.find_indices_1d(xi, xo, method=method)
        if method == "searchsorted":
            # searchsorted is only defined on ascending rows
            got, exp = np.delete(got, 3, axis=0), np.delete(exp, 3, axis=0)
        assert_same(got, exp)


# ---------------------------------------------------------------------------
# 2D point location
# ---------------------------------------------------------------------------


@pytest.mark.parametrize("k", range(6))
def test_locate_known_answers(rg, k):
    c = KNOWN.case(f"loc_{k}")
    g = c.tuple("grid")
    p = c["point"]
    for method, key in (("exhaustive", "brute"), ("secant", "secant"), ("brute", "brute")):
        oi, oj = rg.locate_2d(g, p[:1], p[1:], method=method)
        assert (int(oi[0]), int(oj[0])) == tuple(int(v) for v in c[key]), method


def test_locate_against_oracle(rg):
    c = CURVI.case("curvi129")
    g = c.tuple("ci")
    rng = np.random.default_rng(3)
    px = rng.uniform(-1.3, 1.3, 4000)
    py = rng.uniform(-1.3, 1.3, 4000)
    # points on vertices and edge midpoints of the grid
    px[:50] = g[0][5:55, 7]
    py[:50] = g[1][5:55, 7]
    px[50:100] = 0.5 * (g[0][10, 3:53] + g[0][10, 4:54])
    py[50:100] = 0.5 * (g[1][10, 3:53] + g[1][10, 4:54])
    exp = oracle.locate(g, px, py, "brute")
    for method in ("brute", "exhaustive"):
        got = rg.locate_2d(g, px, py, method=method)
        assert_same(got[0], exp[0])
        assert_same(got[1], exp[1])
    got = rg.locate_2d(g, px, py, method="secant")
    exp = oracle.locate(g, px, py, "secant")
    assert_same(got[0], exp[0])
    assert_same(got[1], exp[1])


@pytest.mark.parametrize("grid", ["rect", "wavy", "rotated"])
def test_locate_outside_points_against_oracle(rg, grid):
    """Points the walk cannot place: outside the grid (in concave pockets of
    the boundary, at exactly the y of boundary vertices, at the extreme y)
    and on the boundary itself, against the oracle's exhaustive locate."""
    from regridding_gb300 import workloads

    n = 41
    if grid == "rect":
        g = workloads.rect_grid(n, -1.0, 1.0)
    elif grid == "wavy":
        a = np.linspace(-1, 1, n)
        x, y = np.meshgrid(a, a, indexing="ij")
        g = (x + 0.08 * np.sin(3 * np.pi * y), y + 0.08 * np.sin(3 * np.pi * x))  # concave boundary, no folds
    else:
        g = workloads.distorted_grid(n, 0.4, 0.03)
    bx = np.concatenate([g[0][:, 0], g[0][-1, :], g[0][::-1, -1], g[0][0, ::-1]])
    by = np.concatenate([g[1][:, 0], g[1][-1, :], g[1][::-1, -1], g[1][0, ::-1]])
    rng = np.random.default_rng(11)
    pts = [
        (bx, by),  # boundary vertices
        (0.5 * (bx[:-1] + bx[1:]), 0.5 * (by[:-1] + by[1:])),  # boundary edge midpoints
        (rng.uniform(-1.6, 1.6, bx.size), by),  # the y of every boundary vertex
        (rng.uniform(-1.6, 1.6, 64), np.full(64, by.min())),
        (rng.uniform(-1.6, 1.6, 64), np.full(64, by.max())),
        (rng.uniform(-1.6, 1.6, 3000), rng.uniform(-1.6, 1.6, 3000)),
        (np.array([5.0, -5.0, 0.0, 0.0]), np.array([0.0, 0.0, 5.0, -5.0])),
    ]
    px = np.concatenate([p[0] for p in pts])
    py = np.concatenate([p[1] for p in pts])
    exp = oracle.locate(g, px, py, "brute")
    got = rg.locate_2d(g, px, py, method="brute")
    assert_same(got[0], exp[0])
    assert_same(got[1], exp[1])
    assert np.sum(exp[0] == np.iinfo(np.int64).max) > 100  # many outside points exercised


def test_find_indices_2d_extension(rg):
    c = CURVI.case("curvi33")
    gi, go = c.tuple("ci"), c.tuple("co")
    i, j = rg.find_indices(gi, go)
    exp = oracle.locate(gi, go[0].ravel(), go[1].ravel(), "brute")
    fill = np.iinfo(np.int64).max
    assert_same(i.ravel(), np.where(exp[0] == fill, fill, exp[0]))
    assert_same(j.ravel(), exp[1])
    with pytest.raises(ValueError):
        rg.find_indices(gi, go, method="searchsorted")


# ---------------------------------------------------------------------------
# benchmark-shaped grids
# ---------------------------------------------------------------------------


@pytest.mark.parametrize("name", ["cfg1", "curvi33", "curvi129"])
def test_curvilinear_weights_bit_exact(rg, name):
    c = CURVI.case(name)
    w = rg.weights(c.tuple("ci"), c.tuple("co"), method="conservative")
    assert_weights_same(w, c.weights())


def test_cfg1_apply(rg):
    c = CURVI.case("cfg1")
    w = rg.weights(c.tuple("ci"), c.tuple("co"), method="conservative")
    res = rg.regrid_from_weights(*w, values_input=c["values_input"])
    assert_same(res, c["result"])
    assert_same(rg.regrid(c.tuple("ci"), c.tuple("co"), values_input=c["values_input"], method="conservative"),
                c["result"])
    f32 = c["values_input"].astype(np.float32)
    fast = rg.regrid_from_weights(*w, values_input=f32, accumulate="fast")
    assert fast.dtype == np.float32
    np.testing.assert_allclose(fast, c["result"], rtol=1e-6, atol=1e-6 * np.abs(c["result"]).max())
    # the upstream in-place float32 output
    out32 = np.empty((8, 48, 48), dtype=np.float32)
    rg.regrid_from_weights(*w, values_input=f32, values_output=out32)
    (ii, oo, vv), = w[0].reshape(-1)
    exp32 = np.empty((8, 48 * 48), dtype=np.float32)
    oracle.apply(ii, oo, vv, f32.reshape(8, -1), 48 * 48, values_output=exp32)
    assert_same(out32.reshape(8, -1), exp32)
    swapped = rg.weights(c.tuple("co"), c.tuple("ci"), weights_input=np.linspace(0.5, 2, 48 * 48).reshape(48, 48),
                         method="conservative")
    (si, so, sv), = swapped[0].reshape(-1)
    assert si.size > 0 and np.all(sv[np.abs(sv) > 1e-12] > 0)


def distorted(n, angle, amp, lo=-1.0, hi=1.0):
    a = np.linspace(lo, hi, n)
    x, y = np.meshgrid(a, a, indexing="ij")
    xr = x * np.cos(angle) - y * np.sin(angle)
    yr = x * np.sin(angle) + y * np.cos(angle)
    xr = xr + amp * np.sin(np.pi * yr)
    yr = yr + amp * np.sin(np.pi * xr)
    return xr, yr


def rect(n, lo, hi):
    a = np.linspace(lo, hi, n)
    return tuple(np.meshgrid(a, a, indexing="ij"))


@pytest.mark.parametrize("n_in,n_out,angle", [(257, 193, 0.25), (513, 385, 0.4), (200, 301, 0.1)])
def test_weights_against_oracle(rg, n_in, n_out, angle):
    gi = distorted(n_in, angle, 0.02)
    go = rect(n_out, -1.05, 1.05)
    rng = np.random.default_rng(42)
    gop = tuple(rng.normal(a, np.ptp(a) * 1e-9) for a in go)
    exp = oracle.weights_conservative_2d(gi, gop)
    dw = rg.build_conservative_2d(gi, gop)
    got = dw.export_numpy()
    for g, e in zip(got, exp):
        assert_same(g, e)
    # apply: exact float64 bit for bit, fast float32 within 1e-6
    import torch

    vals = rng.lognormal(3, 1, (16, n_in - 1, n_in - 1)).astype(np.float32)
    ref = oracle.apply(exp[0], exp[1], exp[2], vals.reshape(16, -1), (n_out - 1) ** 2)
    d_vals = torch.from_numpy(vals.reshape(16, -1)).cuda()
    exact = dw.apply(d_vals).cpu().numpy()
    assert_same(exact, ref)
    fast = dw.apply(d_vals, accumulate="fast").cpu().numpy()
    assert fast.dtype == np.float32
    np.testing.assert_allclose(fast, ref, rtol=1e-6, atol=1e-6 * ref.max())
    # transposed apply against the oracle with swapped indices
    back = dw.apply(torch.from_numpy(ref).cuda(), transpose=True).cpu().numpy()
    ref_t = oracle.apply(exp[1], exp[0], exp[2], ref, (n_in - 1) ** 2)
    np.testing.assert_allclose(back, ref_t, rtol=1e-12, atol=1e-12 * np.abs(ref_t).max())


def test_build_is_deterministic(rg):
    gi = distorted(301, 0.3, 0.03)
    rng = np.random.default_rng(5)
    go = tuple(rng.normal(a, np.ptp(a) * 1e-9) for a in rect(257, -1.1, 1.1))
    a = rg.build_conservative_2d(gi, go).export_numpy()
    b = rg.build_conservative_2d(gi, go).export_numpy()
    for x, y in zip(a, b):
        assert_same(x, y)


def test_large_grid_properties(rg):
    """2048^2 -> 1536^2: size-independent checks (conservation, bounds, symmetry of roles)."""
    import torch

    gi = distorted(2049, 0.3, 0.02)
    go = rect(1537, -1.05, 1.05)
    rng = np.random.default_rng(42)
    go = tuple(rng.normal(a, np.ptp(a) * 1e-9) for a in go)
    dw = rg.build_conservative_2d(gi, go)
    ii, oo, vv = dw.export_numpy()
    assert np.all(np.diff(ii) >= 0)
    area_in = rg.cell_volume(gi, (0, 1)).reshape(-1)
    area_out = rg.cell_volume(go, (0, 1)).reshape(-1)
    overlap = np.bincount(oo, weights=vv * area_in[ii], minlength=area_out.size)
    # each output cell is covered at most once (to rounding of the cancelling sums)
    assert np.all(overlap <= area_out * (1 + 1e-9) + 1e-15)
    # each input cell distributes at most all of itself
    frac = np.bincount(ii, weights=vv, minlength=area_in.size)
    assert np.all(frac <= 1 + 1e-9)
    # interior input cells are fully covered by the larger output grid
    inner = frac.reshape(2048, 2048)[200:-200, 200:-200]
    np.testing.assert_allclose(inner, 1.0, rtol=0, atol=1e-9)
    # apply conserves the covered flux
    vals = torch.ones((2, 2048 * 2048), dtype=torch.float32, device="cuda")
    out = dw.apply(vals).cpu().numpy()
    np.testing.assert_allclose(out[0].sum(), frac.sum(), rtol=1e-9)
    assert frac.sum() > 0.9 * 2048 * 2048


def test_degenerate_grids_report_walk_error(rg):
    """Exactly coincident input and output vertices without the default
    perturbation make the upstream walk cycle forever; the oracle and the
    GPU both stop at their step caps and report it."""
    gi = distorted(65, 0.3, 0.02)
    go = rect(49, -1.05, 1.05)
    with pytest.raises(RuntimeError):
        oracle.sweep_2d(gi, go)
    with pytest.raises(rg.RegridError, match="step cap"):
        rg.build_conservative_2d(gi, go)
    # the library stays usable afterwards
    rng = np.random.default_rng(42)
    gop = tuple(rng.normal(a, np.ptp(a) * 1e-9) for a in go)
    assert rg.build_conservative_2d(gi, gop).nnz > 0


def test_apply_from_host_buffers(rg):
    """rg_apply_host (chunked, three streams) equals the device apply."""
    import ctypes

    import torch
    from regridding_gb300 import _lib

    c = CURVI.case("curvi129")
    w = rg.weights(c.tuple("ci"), c.tuple("co"), method="conservative")
    (ii, oo, vv), = w[0].reshape(-1)
    dw = rg.DeviceWeights.from_coo(ii, oo, vv, 128 * 128, 96 * 96, (96, 96))
    rng = np.random.default_rng(1)
    vals = rng.lognormal(3, 1, (37, 128 * 128)).astype(np.float32)
    ref = dw.apply(torch.from_numpy(vals).cuda(), accumulate="fast").cpu().numpy()
    h_in = torch.from_numpy(vals).pin_memory()
    for chunk in (0, 1, 5, 37, 100):
        h_out = torch.zeros((37, 96 * 96), dtype=torch.float32).pin_memory()
        s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _lib.call("rg_apply_host", dw.handle, ctypes.c_void_p(h_in.data_ptr()), _lib.RG_F32,
                  ctypes.c_void_p(h_out.data_ptr()), _lib.RG_F32, 37, _lib.RG_ACC_FAST, chunk, s)
        torch.cuda.synchronize()
        assert_same(h_out.numpy(), ref)
    # exact float64 output from float64 host input, pageable memory
    v64 = vals.astype(np.float64)
    out64 = np.zeros((37, 96 * 96))
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.call("rg_apply_host", dw.handle, ctypes.c_void_p(v64.ctypes.data), _lib.RG_F64,
              ctypes.c_void_p(out64.ctypes.data), _lib.RG_F64, 37, _lib.RG_ACC_EXACT, 8, s)
    torch.cuda.synchronize()
    assert_same(out64, oracle.apply(ii, oo, vv, v64, 96 * 96))


@pytest.mark.parametrize("chunk", ["0", "1", "3", "7"])
def test_walk_chunking_is_exact(rg, chunk, monkeypatch):
    """Whole-line walks (0) and short chunks (many seats, many repairs) give
    the same bits as the default chunked walk and the oracle."""
    monkeypatch.setenv("RG_SWEEP_CHUNK", chunk)
    c = CURVI.case("curvi33")
    w = rg.weights(c.tuple("ci"), c.tuple("co"), method="conservative")
    assert_weights_same(w, c.weights())
    k = KNOWN.case("c2d_9")  # exact 180-degree rotation: vertices on edges
    w = rg.weights(k.tuple("ci"), k.tuple("co"), method="conservative", perturb=False)
    assert_weights_same(w, k.weights())
    gi = distorted(257, 0.25, 0.02)
    rng = np.random.default_rng(42)
    gop = tuple(rng.normal(a, np.ptp(a) * 1e-9) for a in rect(193, -1.05, 1.05))
    exp = oracle.weights_conservative_2d(gi, gop)
    got = rg.build_conservative_2d(gi, gop).export_numpy()
    for g, e in zip(got, exp):
        assert_same(g, e)


def _local_coo(rng, n0_in, n1_in, n0_out, n1_out, per_row=(1, 9), empty=0.0, spread=None):
    """Entries of a 2D-to-2D weights matrix whose output cell (i, j) reads a
    small neighbourhood of the corresponding input cell (or, with `spread`,
    `spread` random cells anywhere in the input)."""
    ii, oo = [], []
    for o in range(n0_out * n1_out):
        if rng.random() < empty:
            continue
        i, j = divmod(o, n1_out)
        ci = int(i * n0_in / n0_out)
        cj = int(j * n1_in / n1_out)
        if spread:
            cells = rng.choice(n0_in * n1_in, size=spread, replace=False)
        else:
            k = int(rng.integers(*per_row))
            di = rng.integers(-1, 2, k)
            dj = rng.integers(-2, 3, k)
            cells = np.unique(np.clip(ci + di, 0, n0_in - 1) * n1_in + np.clip(cj + dj, 0, n1_in - 1))
        ii.extend(cells.tolist())
        oo.extend([o] * len(cells))
    ii = np.asarray(ii, dtype=np.int64)
    oo = np.asarray(oo, dtype=np.int64)
    vv = rng.uniform(0.1, 1.0, ii.size)
    return ii, oo, vv


@pytest.mark.parametrize(
    "case",
    ["vec", "vec_tail4", "scalar_odd", "unaligned", "long_lists", "huge_tile", "no_shape", "empty_rows",
     "tma", "tma_some_far", "tma_all_far"])
@pytest.mark.parametrize("stack", [1, 7, 64])
def test_fast_apply_paths(rg, case, stack):
    """Every branch of the float32 fast apply against the oracle's float64
    apply: sector lists (n_in % 8 == 0 and == 4, where the last sector's
    second half lies past the slice), cell lists (n_in % 4 != 0, unaligned
    input), tiles whose lists overflow into the direct gathers, unknown
    output shape (row tiles), rows without entries, and the tensor-copy
    staging (input shape known: boxes for all tiles, for all but a few, or
    footprints too scattered for a box).  float32 accumulation with FMA is
    checked against its forward error bound."""
    import torch

    from regridding_gb300._device import DeviceWeights

    rng = np.random.default_rng([len(case), sum(map(ord, case)), stack])
    n0_in, n1_in, n0_out, n1_out = 40, 48, 30, 37
    kw = {}
    if case == "scalar_odd":
        n1_in = 47
    if case == "long_lists":
        kw = {"spread": 6}
    if case == "huge_tile":
        n0_in, n1_in = 100, 64
    if case == "empty_rows":
        kw = {"empty": 0.4}
    if case == "tma_all_far":
        kw = {"spread": 3}
    ii, oo, vv = _local_coo(rng, n0_in, n1_in, n0_out, n1_out, **kw)
    n_in = n0_in * n1_in
    if case == "tma_some_far":
        # a far-away cell in 4 rows: those tiles' footprints exceed the box
        # and take the direct gathers; the rest are staged by tensor copies
        key = np.unique(np.concatenate([oo * n_in + ii, np.array([5, 200, 611, 1000]) * n_in + [1913, 3, 960, 47]]))
        oo, ii = key // n_in, key % n_in
        vv = rng.uniform(0.1, 1.0, ii.size)
    if case == "vec_tail4":
        n_in = 1796  # n_in % 8 == 4; make sure the last cell is read
        ii = np.minimum(ii, n_in - 1)
        ii[-1] = n_in - 1
        key = np.unique(oo * n_in + ii)
        oo, ii = key // n_in, key % n_in
        vv = rng.uniform(0.1, 1.0, ii.size)
    if case == "huge_tile":
        # one output cell reading 5000 inputs: its tile has more entries than
        # the tile sorter holds and takes the direct gathers
        extra = rng.choice(n_in, size=5000, replace=False)
        keep = oo != 5
        ii = np.concatenate([ii[keep], extra])
        oo = np.concatenate([oo[keep], np.full(5000, 5)])
        vv = np.concatenate([vv[keep], rng.uniform(0.1, 1.0, 5000) / 1000])
    n_out = n0_out * n1_out
    shape = None if case == "no_shape" else (n0_out, n1_out)
    dw = DeviceWeights.from_coo(ii, oo, vv, n_in, n_out, shape)
    if case.startswith("tma"):
        from regridding_gb300 import _lib

        _lib.call("rg_weights_set_input_shape", dw.handle, n0_in, n1_in)
    vals = rng.uniform(0.5, 2.0, (stack, n_in)).astype(np.float32)
    if case == "unaligned":
        buf = torch.empty(stack * n_in + 1, dtype=torch.float32, device="cuda")
        d_vals = buf[1:].view(stack, n_in)
        d_vals.copy_(torch.from_numpy(vals))
        assert d_vals.data_ptr() % 16 != 0
    else:
        d_vals = torch.from_numpy(vals).cuda()
    got = dw.apply(d_vals, accumulate="fast").cpu().numpy()
    exp = oracle.apply(ii, oo, vv, vals.astype(np.float64), n_out)
    assert got.dtype == np.float32 and got.shape == (stack, n_out)
    # forward error bound of a float32 FMA chain of k terms with weights
    # rounded to float32: (k + 2) u sum|w x|, u = 2^-24
    k = np.bincount(oo, minlength=n_out)
    bound = (k + 2) * 2.0**-24 * oracle.apply(ii, oo, np.abs(vv), np.abs(vals).astype(np.float64), n_out)
    assert np.all(np.abs(got - exp) <= bound), np.max(np.abs(got - exp) / np.maximum(bound, 1e-300))
    if case == "empty_rows":
        empty = np.setdiff1d(np.arange(n_out), oo)
        assert empty.size > 0 and np.all(got[:, empty] == 0)
    # applying twice (lists already built) gives the same bits
    again = dw.apply(d_vals, accumulate="fast").cpu().numpy()
    assert_same(again, got)
    if stack > 1:
        # fewer slices than the tuned stage size (the warp-staged kernel takes over)
        one = dw.apply(d_vals[:1].contiguous(), accumulate="fast").cpu().numpy()
        assert_same(one, got[:1])
    # the exact apply of the float32 stack: the upstream float64 result bit for bit
    exact = dw.apply(d_vals, accumulate="exact").cpu().numpy()
    assert exact.dtype == np.float64
    assert_same(exact, oracle.apply(ii, oo, vv, vals, n_out))
    from regridding_gb300 import _lib

    _lib.call("rg_weights_check", dw.handle, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


@pytest.mark.parametrize("kind", ["multilinear", "conservative_coarse"])
def test_row_kernel_long_stacks(rg, kind):
    """Weights with a short input axis over a long stack take the row kernel
    (whole slices staged by bulk copies); its results are within the float32
    bound of the oracle and bit-identical to the same weights over a short
    stack (warp-staged kernel, same per-row order).  Rows longer than the
    kernel holds (coarse conservative output) take the other kernels."""
    import torch

    from regridding_gb300._device import DeviceWeights

    rng = np.random.default_rng(31)
    x_in = np.sort(rng.uniform(0, 1, 512))
    if kind == "multilinear":
        x_out = np.sort(rng.uniform(x_in[0], x_in[-1], 400))
        w, _, _ = rg.weights(x_in, x_out, method="multilinear")
    else:
        x_out = np.linspace(x_in[0], x_in[-1], 41)  # ~13 input cells per output cell
        w, _, _ = rg.weights(x_in, x_out, method="conservative")
    ii, oo, vv = w[()] if w.shape == () else w.reshape(-1)[0]
    n_in = 512 if kind == "multilinear" else 511  # conservative: 511 cells
    n_out = 400 if kind == "multilinear" else 40
    dw = DeviceWeights.from_coo(ii, oo, vv, n_in, n_out)
    vals = rng.uniform(0.5, 2.0, (700, n_in)).astype(np.float32)
    d_vals = torch.from_numpy(vals).cuda()
    got = dw.apply(d_vals, accumulate="fast").cpu().numpy()
    short = dw.apply(d_vals[:37].contiguous(), accumulate="fast").cpu().numpy()
    assert_same(short, got[:37])
    exp = oracle.apply(ii, oo, vv, vals.astype(np.float64), n_out)
    k = np.bincount(oo, minlength=n_out)
    bound = (k + 2) * 2.0**-24 * oracle.apply(ii, oo, np.abs(vv), np.abs(vals).astype(np.float64), n_out)
    assert np.all(np.abs(got - exp) <= bound)
    from regridding_gb300 import _lib

    _lib.call("rg_weights_check", dw.handle, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def test_copy_from_host_and_attributes(rg):
    """rg_copy_from_host (a kernel reading pageable host memory where the
    device allows it, else a copy-engine copy) copies every byte, aligned or
    not; rg_device_attributes reports the SM count."""
    import ctypes

    import torch

    from regridding_gb300 import _device, _lib

    attrs = np.zeros(6, np.int64)
    _lib.call("rg_device_attributes", ctypes.c_void_p(attrs.ctypes.data), 6)
    assert attrs[0] == torch.cuda.get_device_properties(0).multi_processor_count
    rng = np.random.default_rng(11)
    for n in (1, 7, 8, 4096 + 3, 3 << 20):
        src = rng.integers(0, 256, n + 1, dtype=np.uint8)
        for off in (0, 1):
            d = torch.zeros(n, dtype=torch.uint8, device="cuda")
            _lib.call("rg_copy_from_host", _device.ptr(d), ctypes.c_void_p(src.ctypes.data + off), n,
                      _device.stream())
            np.testing.assert_array_equal(d.cpu().numpy(), src[off:off + n])
    big = rng.normal(0, 1, (1000, 1000))
    np.testing.assert_array_equal(_device.download(_device.upload(big)), big)


BOX_CONFIGS = ["4,2,0", "4,2,4", "4,3,4", "2,3,4", "2,4,4", "8,2,0", "4,3,0"]


@pytest.mark.parametrize("stack", [1, 7, 64])
def test_box_configs_agree(rg, stack, monkeypatch):
    """Every configuration of the tensor-copy apply (slices per stage,
    stages, register cap), forced in turn, gives the same float32 result bit
    for bit (each output's FMA chain is the same), with some patches on the
    direct path, and matches the oracle's bound."""
    import torch

    from regridding_gb300 import _lib
    from regridding_gb300._device import DeviceWeights

    rng = np.random.default_rng([99, stack])
    n0_in, n1_in, n0_out, n1_out = 64, 96, 48, 60
    ii, oo, vv = _local_coo(rng, n0_in, n1_in, n0_out, n1_out)
    n_in, n_out = n0_in * n1_in, n0_out * n1_out
    key = np.unique(np.concatenate([oo * n_in + ii, np.array([7, 900]) * n_in + [n_in - 5, 11]]))
    oo, ii = key // n_in, key % n_in
    vv = rng.uniform(0.1, 1.0, ii.size)
    vals = rng.uniform(0.5, 2.0, (stack, n_in)).astype(np.float32)
    d_vals = torch.from_numpy(vals).cuda()
    results = []
    for cfg in BOX_CONFIGS:
        monkeypatch.setenv("RG_APPLY_BOX_CONFIG", cfg)
        dw = DeviceWeights.from_coo(ii, oo, vv, n_in, n_out, (n0_out, n1_out))
        _lib.call("rg_weights_set_input_shape", dw.handle, n0_in, n1_in)
        results.append(dw.apply(d_vals, accumulate="fast").cpu().numpy())
        dw.free()
    for cfg, got in zip(BOX_CONFIGS[1:], results[1:]):
        np.testing.assert_array_equal(got, results[0], err_msg=cfg)
    exp = oracle.apply(ii, oo, vv, vals.astype(np.float64), n_out)
    k = np.bincount(oo, minlength=n_out)
    bound = (k + 2) * 2.0**-24 * oracle.apply(ii, oo, np.abs(vv), np.abs(vals).astype(np.float64), n_out)
    assert np.all(np.abs(results[0] - exp) <= bound)
