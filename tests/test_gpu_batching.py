"""Batched builds and graph-replayed applies on the GPU: every pair of a
batch gets bit for bit the weights of its own build (and of the oracle),
a degenerate pair fails alone, sub-batch splits do not change results, and
a replayed CUDA graph of applies writes exactly what the eager applies do."""

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


def uneven_pairs(n=12, seed=21):
    from regridding_gb300 import workloads

    rng = np.random.default_rng(seed)
    return [workloads.grid_pair(rng, workloads.log_uniform_side(rng, 8, 72)) for _ in range(n)]


def same_weights(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def test_batch_equals_single_builds_and_oracle(torch):
    import regridding_gb300 as rg
    from regridding_gb300 import batching

    pairs = uneven_pairs()
    built = batching.build_batch(pairs)
    for k, ((gi, go), dw) in enumerate(zip(pairs, built)):
        assert isinstance(dw, rg._device.DeviceWeights), dw
        got = dw.export_numpy()
        assert same_weights(got, rg.build_conservative_2d(gi, go).export_numpy()), k
        if k < 4:
            assert same_weights(got, oracle.weights_conservative_2d(gi, go)), k


def test_sub_batches_and_failed_pair(torch):
    import regridding_gb300 as rg
    from regridding_gb300 import batching, workloads

    pairs = uneven_pairs(8, seed=22)
    # an unperturbed pair sharing the vertex (0, 0): the upstream sweep
    # cycles around it (the oracle shows it); the build stops at its step cap
    bad = (workloads.distorted_grid(65, 0.3, 0.02), workloads.rect_grid(49, -1.05, 1.05))
    with pytest.raises(RuntimeError):
        oracle.sweep_2d(*bad)
    pairs.insert(3, bad)
    whole = batching.build_batch(pairs)
    split = batching.build_batch(pairs, max_cells=3000)  # several sub-batches
    assert isinstance(whole[3], rg.RegridError) and isinstance(split[3], rg.RegridError)
    for k in range(len(pairs)):
        if k == 3:
            continue
        assert same_weights(whole[k].export_numpy(), split[k].export_numpy()), k
        assert same_weights(whole[k].export_numpy(), rg.build_conservative_2d(*pairs[k]).export_numpy()), k


@pytest.mark.parametrize("chunk", [0, 5, 32])
def test_chunk_length_does_not_change_weights(torch, chunk):
    import regridding_gb300 as rg
    from regridding_gb300 import _lib, batching

    pairs = uneven_pairs(6, seed=23)
    ref = [rg.build_conservative_2d(gi, go).export_numpy() for gi, go in pairs]
    try:
        _lib.call("rg_set_sweep_chunk", chunk)
        got = batching.build_batch(pairs)
    finally:
        _lib.call("rg_set_sweep_chunk", 32)
    for r, w in zip(ref, got):
        assert same_weights(r, w.export_numpy())


@pytest.mark.parametrize("branches", [1, 3, 8])
def test_apply_graph_replays_the_eager_applies(torch, branches):
    """The graph (its applies in 1, 3 or 8 parallel chains) gives the eager
    applies' results bit for bit, and reads new inputs at every replay."""
    from regridding_gb300 import batching

    pairs = uneven_pairs(10, seed=24)
    built = batching.build_batch(pairs)
    rng = np.random.default_rng(5)
    items = []
    for (gi, go), dw in zip(pairs, built):
        stack = int(rng.choice((1, 4, 16)))
        v = torch.from_numpy(rng.poisson(50, (stack, dw.n_in)).astype(np.float32)).cuda()
        o = torch.empty((stack, dw.n_out), dtype=torch.float32, device="cuda")
        items.append((dw, v, o))
    graph = batching.ApplyGraph(items, branches=branches)
    assert sorted(k for c in graph.chains for k in c) == list(range(len(items)))
    eager = [dw.apply(v, accumulate="fast").cpu().numpy() for dw, v, _ in items]
    for _, _, o in items:
        o.zero_()
    graph.replay()
    torch.cuda.synchronize()
    for (_, _, o), e in zip(items, eager):
        np.testing.assert_array_equal(o.cpu().numpy(), e)
    # new inputs in the same tensors: the replay reads them
    for dw, v, _ in items:
        v.mul_(2.0)
    graph.replay()
    torch.cuda.synchronize()
    for (dw, v, o), e in zip(items, eager):
        np.testing.assert_allclose(o.cpu().numpy(), 2 * e, rtol=1e-6)


def test_autotune_sweep_chunk(torch):
    from regridding_gb300 import _lib, batching

    pairs = uneven_pairs(4, seed=25)
    try:
        t = batching.autotune_sweep_chunk(pairs, candidates=(16, 32))
        assert set(t) == {16, 32} and all(v > 0 for v in t.values())
    finally:
        _lib.call("rg_set_sweep_chunk", 32)
