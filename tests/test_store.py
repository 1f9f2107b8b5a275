"""On-disk weights: the file format round trip (bit-exact, read-only
memory-mapped elements, empty elements, object arrays of any shape), key
stability and equivalence rules, the directory cache's hit/miss/eviction
logic with a stand-in builder, and on the GPU the cache around the real
weights() and the serving path's disk loads."""

import os
import pickle

import numpy as np
import pytest

import fixtures

KNOWN = fixtures.load("known_answers.npz")


def layout(rng, shape=(2, 3), n_in=50, n_out=40):
    array = np.empty(shape, dtype=object)
    for idx in np.ndindex(*shape):
        nnz = int(rng.integers(0, 30))
        array[idx] = (np.sort(rng.integers(0, n_in, nnz)), rng.integers(0, n_out, nnz), rng.normal(0, 1, nnz))
    return array, (n_in,), (n_out,)


@pytest.mark.parametrize("mmap", [True, False])
@pytest.mark.parametrize("shape", [(), (4,), (2, 3), (0,)])
def test_round_trip(tmp_path, shape, mmap):
    from regridding_gb300 import store

    rng = np.random.default_rng(1)
    w = layout(rng, shape)
    p = tmp_path / "w.rgw"
    size = store.save_weights(p, w, {"note": "x"})
    assert size == os.path.getsize(p) and size % store.ALIGN == 0
    array, si, so = store.load_weights(p, mmap=mmap)
    assert array.shape == w[0].shape and (si, so) == (w[1], w[2])
    for idx in np.ndindex(*shape):
        for got, exp in zip(array[idx], w[0][idx]):
            assert not got.flags.writeable
            np.testing.assert_array_equal(got, exp)
            assert got.dtype == (np.float64 if exp.dtype.kind == "f" else np.int64)
    assert store.read_header(p)["meta"] == {"note": "x"}


def test_upstream_layout_round_trip(tmp_path):
    """A saved layout produced by the upstream package survives the file
    and pickles afterwards (the upstream contract)."""
    from regridding_gb300 import store

    c = KNOWN.case(next(n for n in KNOWN.names("c2d_") if "weights" in KNOWN.case(n).meta))
    w = c.weights("weights")
    store.save_weights(tmp_path / "u.rgw", w)
    got = store.load_weights(tmp_path / "u.rgw")
    for idx in np.ndindex(*w[0].shape):
        for a, b in zip(got[0][idx], w[0][idx]):
            np.testing.assert_array_equal(a, b)
    again = pickle.loads(pickle.dumps(got))
    np.testing.assert_array_equal(again[0].reshape(-1)[0][2], w[0].reshape(-1)[0][2])


def test_not_a_weights_file(tmp_path):
    from regridding_gb300 import store

    p = tmp_path / "bad.rgw"
    p.write_bytes(b"hello" * 20)
    with pytest.raises(ValueError, match="not a weights file"):
        store.load_weights(p)


def test_truncated_or_corrupt_files_are_rejected(tmp_path):
    """A short file, element offsets that do not add up, and a header whose
    arrays lie past the end raise ValueError (which the cache treats as a
    miss), instead of returning silently truncated elements."""
    from regridding_gb300 import store

    rng = np.random.default_rng(3)
    w = layout(rng, (5,))
    p = tmp_path / "w.rgw"
    store.save_weights(p, w)
    full = p.read_bytes()
    header = store.read_header(p)
    short = tmp_path / "short.rgw"
    short.write_bytes(full[: header["offsets"][3] + 8])  # values cut off
    with pytest.raises(ValueError, match="truncated"):
        store.load_weights(short)
    bad = bytearray(full)
    s_off = header["offsets"][0]
    bad[s_off + 8: s_off + 16] = (10**6).to_bytes(8, "little")  # the second element's end offset
    corrupt = tmp_path / "corrupt.rgw"
    corrupt.write_bytes(bytes(bad))
    with pytest.raises(ValueError, match="offsets"):
        store.load_weights(corrupt)
    cache = store.WeightsDiskCache(tmp_path / "c")
    os.replace(short, cache.path("k1"))
    assert cache.get("k1") is None and cache.misses == 1


def test_cache_ignores_files_of_another_build(tmp_path, monkeypatch):
    """Keys and file headers carry the library version and weights revision:
    a file written by another build is a miss, never a hit."""
    from regridding_gb300 import store

    rng = np.random.default_rng(4)
    cache = store.WeightsDiskCache(tmp_path)
    cache.put("k", layout(rng, (2,)))
    assert cache.get("k") is not None
    assert store.read_header(cache.path("k"))["build"] == store.build_tag()
    monkeypatch.setattr(store, "WEIGHTS_REVISION", store.WEIGHTS_REVISION + 1)
    assert cache.get("k") is None
    gi = (np.linspace(0, 1, 5),)
    k2 = store.weights_key(gi, gi)
    monkeypatch.setattr(store, "WEIGHTS_REVISION", store.WEIGHTS_REVISION + 1)
    assert store.weights_key(gi, gi) != k2


def test_key_rules():
    from regridding_gb300 import store

    rng = np.random.default_rng(2)
    gi = (rng.random((5, 6)), rng.random((5, 6)))
    go = (rng.random((4, 4)), rng.random((4, 4)))
    k = store.weights_key(gi, go, method="conservative")
    assert k == store.weights_key(gi, go, method="conservative", perturb=True, seed=42)
    assert k == store.weights_key(gi, go, method="conservative", bounds="nan")  # bounds: multilinear only
    assert k != store.weights_key(gi, go, method="conservative", seed=7)
    assert k != store.weights_key(gi, go, method="multilinear")
    assert k != store.weights_key(gi, go, method="conservative", weights_input=np.ones((4, 5)))
    assert store.weights_key(gi, go, method="conservative", perturb=False, seed=1) == \
        store.weights_key(gi, go, method="conservative", perturb=False, seed=2)
    assert store.weights_key(gi, go, seed=np.random.default_rng(0)) is None
    go2 = (go[0].copy(), go[1].copy())
    go2[1][0, 0] += 1e-12
    assert k != store.weights_key(gi, go2, method="conservative")


def test_cache_hits_misses_eviction(tmp_path, monkeypatch):
    from regridding_gb300 import _weights, store

    calls = []

    def fake_weights(ci, co, **kw):
        calls.append(kw)
        rng = np.random.default_rng(len(calls))
        return layout(rng, ())

    monkeypatch.setattr(_weights, "weights", fake_weights)
    cache = store.WeightsDiskCache(tmp_path / "c")
    rng = np.random.default_rng(3)
    grids = [((rng.random(9),), (rng.random(7),)) for _ in range(3)]
    first = cache.weights(*grids[0], method="multilinear")
    again = cache.weights(*grids[0], method="multilinear")
    assert len(calls) == 1 and cache.hits == 1 and cache.misses == 1 and cache.writes == 1
    for a, b in zip(first[0][()], again[0][()]):
        np.testing.assert_array_equal(a, b)
    cache.weights(*grids[1], method="multilinear")
    cache.weights(*grids[0], method="multilinear", seed=np.random.default_rng(0))  # not cacheable: builds
    assert len(calls) == 3
    sizes = [e[1] for e in cache.entries()]
    bounded = store.WeightsDiskCache(tmp_path / "c", max_bytes=sizes[0] + 1)
    os.utime(cache.path(store.weights_key(*grids[0], method="multilinear")), (1, 1))  # the oldest
    bounded.trim()
    left = [os.path.basename(e[2]) for e in bounded.entries()]
    assert len(left) == 1 and bounded.evictions == 1
    assert left[0].startswith(store.weights_key(*grids[1], method="multilinear"))


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


@pytest.mark.gpu
def test_gpu_cache_around_weights(torch, tmp_path):
    import regridding_gb300 as rg
    from regridding_gb300 import store, workloads

    gi = workloads.distorted_grid(33, 0.0, 0.02)
    go = workloads.rect_grid(25, -0.9, 0.9)
    cache = store.WeightsDiskCache(tmp_path)
    w1 = cache.weights(gi, go, method="conservative")
    w2 = cache.weights(gi, go, method="conservative")
    exp = rg.weights(gi, go, method="conservative")
    for w in (w1, w2):
        for a, b in zip(w[0][()], exp[0][()]):
            np.testing.assert_array_equal(a, b)
    vals = np.random.default_rng(4).normal(0, 1, (3, 32, 32))
    np.testing.assert_array_equal(rg.regrid_from_weights(*w2, vals), rg.regrid_from_weights(*exp, vals))
    assert cache.hits == 1 and cache.writes == 1


@pytest.mark.gpu
def test_gpu_server_disk_cache(torch, tmp_path):
    """A second server finds the weights the first one wrote, and its
    results are the same; the files are those of the cache's weights()."""
    from regridding_gb300 import store, workloads
    from regridding_gb300.serving import RegridServer

    gi = workloads.distorted_grid(65, 0.0, 0.02)
    go = workloads.rect_grid(49, -0.9, 0.9)
    vals = torch.from_numpy(np.random.default_rng(5).normal(0, 1, (2, 64 * 64)).astype(np.float32))
    cache = store.WeightsDiskCache(tmp_path)
    outs = []
    for _ in range(2):
        server = RegridServer(hbm_budget=4e9, slots=2, disk_cache=cache)
        try:
            outs.append(server.submit(gi, go, vals).result(timeout=120))
            server.backend.flush()
            loads = server.backend.disk_loads
        finally:
            server.close()
    assert loads == 1 and cache.writes == 1
    np.testing.assert_array_equal(outs[0].numpy(), outs[1].numpy())
    assert store.weights_key(gi, go, method="conservative") is not None
    assert cache.get(store.weights_key(gi, go, method="conservative")) is not None


def test_file_backed_arrays_are_recognised(tmp_path):
    """Memory-mapped saved weights and shared-memory arrays are uploaded by
    the copy engines, not read by a kernel (their pages may not be
    resident); ordinary arrays and views of them are not file-backed."""
    from multiprocessing import shared_memory

    from regridding_gb300 import _device, store

    w = layout(np.random.default_rng(4), (2,))
    store.save_weights(tmp_path / "w.rgw", w)
    ii = store.load_weights(tmp_path / "w.rgw")[0][1][0]
    assert _device._file_backed(np.ascontiguousarray(ii))
    sm = shared_memory.SharedMemory(create=True, size=800)
    try:
        a = np.ndarray((100,), dtype=np.float64, buffer=sm.buf)
        assert _device._file_backed(a)
        del a
    finally:
        sm.close()
        sm.unlink()
    b = np.arange(10.0)
    assert not _device._file_backed(b) and not _device._file_backed(b[2:5])
