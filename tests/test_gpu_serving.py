"""The served form on the GPU: every result of a mixed, concurrently
submitted stream equals the same request run alone (bit for bit; the batched
apply computes each slice with the same per-row sums), the fast results are
within the float32 forward error bound of the oracle, and exact-mode results
are bit-identical to the oracle's float64 apply of the oracle's weights."""

import threading

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


def stream_requests(n=36, seed=3):
    from regridding_gb300 import workloads

    rng = np.random.default_rng(seed)
    pairs = [workloads.grid_pair(rng, s) for s in (20, 33, 48, 64, 96)]
    reqs = []
    for i in range(n):
        k = int(rng.integers(len(pairs))) if i % 4 else len(pairs) - 1 - (i // 4) % len(pairs)
        stack = int(rng.choice((1, 3, 8)))
        gi, go = pairs[k]
        n_in = (gi[0].shape[0] - 1) * (gi[0].shape[1] - 1)
        vals = rng.lognormal(3, 1, (stack, n_in)).astype(np.float32)
        reqs.append((k, pairs[k], vals))
    return pairs, reqs


def fast_bound(ii, oo, vv, vals, n_out):
    k = np.bincount(oo, minlength=n_out)
    return (k + 2) * 2.0**-24 * oracle.apply(ii, oo, np.abs(vv), np.abs(vals).astype(np.float64), n_out)


def test_mixed_stream_equals_alone(torch):
    from regridding_gb300.serving import RegridServer, regrid_plain

    pairs, reqs = stream_requests()
    alone = [regrid_plain(gi_go[0], gi_go[1], vals).numpy().copy() for _, gi_go, vals in reqs]
    results = [None] * len(reqs)
    with RegridServer(hbm_budget=4e9, slots=4, max_batch_stack=16) as srv:
        def client(idx):
            futs = [(i, srv.submit(reqs[i][1][0], reqs[i][1][1], reqs[i][2])) for i in idx]
            for i, f in futs:
                results[i] = f.result(120)

        threads = [threading.Thread(target=client, args=(list(range(c, len(reqs), 3)),)) for c in range(3)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        st = srv.stats()
    for got, exp in zip(results, alone):
        np.testing.assert_array_equal(np.asarray(got), exp)
    assert st["builds"] == len(pairs)  # every grid built once, then served from the cache
    assert st["batches"] < len(reqs)  # some requests shared an apply
    # against the oracle: weights of each grid pair, then the float32 bound
    from regridding_gb300 import workloads

    # the server jitters output grids as weights() does by default
    w = {k: oracle.weights_conservative_2d(pairs[k][0], workloads.perturb(pairs[k][1])) for k in range(len(pairs))}
    for (k, (gi, go), vals), got in zip(reqs, results):
        ii, oo, vv = w[k]
        n_out = (go[0].shape[0] - 1) * (go[0].shape[1] - 1)
        exp = oracle.apply(ii, oo, vv, vals.astype(np.float64), n_out)
        assert np.all(np.abs(np.asarray(got) - exp) <= fast_bound(ii, oo, vv, vals, n_out))


def test_exact_mode_is_bit_identical_to_oracle(torch):
    from regridding_gb300.serving import RegridServer

    pairs, reqs = stream_requests(n=12, seed=4)
    with RegridServer(hbm_budget=4e9, slots=3, accumulate="exact") as srv:
        futs = [srv.submit(gi, go, vals) for _, (gi, go), vals in reqs]
        results = [f.result(120) for f in futs]
    from regridding_gb300 import workloads

    for (k, (gi, go), vals), got in zip(reqs, results):
        ii, oo, vv = oracle.weights_conservative_2d(gi, workloads.perturb(go))
        n_out = (go[0].shape[0] - 1) * (go[0].shape[1] - 1)
        got = np.asarray(got)
        assert got.dtype == np.float64
        np.testing.assert_array_equal(got, oracle.apply(ii, oo, vv, vals, n_out))


def test_budget_evicts_and_still_serves(torch):
    from regridding_gb300.serving import RegridServer, regrid_plain

    pairs, reqs = stream_requests(n=20, seed=5)
    # room for only a couple of grids' weights at a time: the cache must evict
    with RegridServer(hbm_budget=6e6, slots=2, cache_bytes=3e5) as srv:
        futs = [srv.submit(gi, go, vals) for _, (gi, go), vals in reqs]
        results = [f.result(120) for f in futs]
        st = srv.stats()
    assert st["evictions"] > 0 and st["peak_bytes"] <= 6e6
    for (_, (gi, go), vals), got in zip(reqs, results):
        np.testing.assert_array_equal(np.asarray(got), regrid_plain(gi, go, vals).numpy())


@pytest.mark.parametrize("accumulate", ["fast", "exact"])
def test_large_pinned_request_is_pipelined_and_equal(torch, accumulate):
    """A request whose stack in pinned host memory reaches the pipelining size
    goes through rg_apply_host (chunks copied in, applied and copied out on
    three streams); its result equals the device apply of the same weights,
    and a batched apply of the same grid (the unpipelined path) slice for
    slice."""
    from regridding_gb300 import workloads
    from regridding_gb300._device import build_conservative_2d
    from regridding_gb300.serving import GpuBackend, RegridServer

    rng = np.random.default_rng(12)
    gi, go = workloads.grid_pair(rng, 1024)
    n_in = (gi[0].shape[0] - 1) * (gi[0].shape[1] - 1)
    n_out = (go[0].shape[0] - 1) * (go[0].shape[1] - 1)
    stack = GpuBackend.PIPELINE_BYTES // (4 * n_in) + 2
    vals = torch.empty((stack, n_in), dtype=torch.float32, pin_memory=True)
    vals.copy_(torch.from_numpy(rng.lognormal(3, 1, (stack, n_in)).astype(np.float32)))
    odt = torch.float32 if accumulate == "fast" else torch.float64
    out = torch.empty((stack, n_out), dtype=odt, pin_memory=True)
    small = vals[:2].clone()  # not pinned: the ordinary path
    with RegridServer(hbm_budget=8e9, slots=2, accumulate=accumulate, perturb=False) as srv:
        assert srv.backend._pipelined([type("R", (), {"values": vals, "out": out})()], None)
        got = srv.submit(gi, go, vals, out=out).result(120)
        got_small = srv.submit(gi, go, small).result(120)
    dw = build_conservative_2d(gi, go)
    try:
        exp = dw.apply(vals.cuda(), accumulate=accumulate).cpu()
    finally:
        dw.free()
    assert got.data_ptr() == out.data_ptr()
    np.testing.assert_array_equal(got.numpy(), exp.numpy())
    np.testing.assert_array_equal(np.asarray(got_small), exp[:2].numpy())
