"""Host logic of the served form (no GPU): the weights LRU, admission by
device footprint, continuous batching of requests for the same grid, error
propagation and shutdown, driven through a fake backend whose "weights" are
small dense numpy matrices."""

import threading
import time

import numpy as np
import pytest

from regridding_gb300.serving import RegridServer, WeightsLRU


class FakeBackend:
    def __init__(self, build_delay=0.0, run_delay=0.0, fail_build=(), gate=None):
        self.lock = threading.Lock()
        self.build_delay = build_delay
        self.run_delay = run_delay
        self.fail_build = set(fail_build)
        self.gate = gate
        self.builds = []
        self.batches = []
        self.freed = []
        self.active = 0
        self.max_active = 0

    def make_slot(self, i):
        return i

    def prepare(self, values, out, n_in, n_out):
        v = np.asarray(values, dtype=np.float64).reshape(-1, n_in)
        o = np.empty((v.shape[0], n_out)) if out is None else out.reshape(v.shape[0], n_out)
        return v, o

    def request_bytes(self, req):
        return req.stack * (req.n_in + req.n_out) * 8

    def build_bytes(self, req):
        # scratch plus the weights the build leaves behind (the real backend's
        # per-cell estimate also covers both)
        return 100 * (req.n_in + req.n_out) + 8 * req.n_in * req.n_out

    @staticmethod
    def matrix(key, n_in, n_out):
        rng = np.random.default_rng(abs(hash(key)) % 2**32)
        return rng.random((n_out, n_in))

    def build(self, slot, req):
        with self.lock:
            self.builds.append(req.key)
        if req.key in self.fail_build:
            raise RuntimeError("build failed")
        time.sleep(self.build_delay)
        m = self.matrix(req.key, req.n_in, req.n_out)
        return m, m.nbytes

    def run(self, slot, m, reqs):
        with self.lock:
            self.active += 1
            self.max_active = max(self.max_active, self.active)
            self.batches.append([r.key for r in reqs])
        if self.gate is not None:
            self.gate.wait(5)
        time.sleep(self.run_delay)
        for r in reqs:
            r.out[:] = r.values @ m.T
        with self.lock:
            self.active -= 1

    def free(self, m):
        with self.lock:
            self.freed.append(m.shape)


def grids(n, m):
    """Vertex grids with n x n input and m x m output cells (contents unused)."""
    gi = np.meshgrid(np.linspace(0, 1, n + 1), np.linspace(0, 1, n + 1), indexing="ij")
    go = np.meshgrid(np.linspace(0, 1, m + 1), np.linspace(0, 1, m + 1), indexing="ij")
    return tuple(gi), tuple(go)


def test_lru_order_refs_and_eviction():
    freed = []
    c = WeightsLRU(100, free=freed.append)
    c.insert("a", "A", 40)
    c.insert("b", "B", 40)
    c.release("a")
    c.release("b")
    assert c.acquire("a") == "A"  # a is now the most recent, and referenced
    c.insert("c", "C", 40)  # over capacity: b (oldest unreferenced) goes
    assert freed == ["B"] and "b" not in c and c.used == 80
    c.release("c")
    c.insert("d", "D", 70)  # a is referenced: only c can go, and the cache stays over
    assert "a" in c and "c" not in c and c.used == 110
    c.release("a")
    c.release("d")
    assert c.used <= 100 and "d" in c  # a evicted once released
    assert c.acquire("zz") is None and c.misses == 1
    c.shrink_by(1000)
    assert c.used == 0 and len(c) == 0


def test_results_and_batching_of_one_grid():
    gate = threading.Event()
    be = FakeBackend(gate=gate)
    gi, go = grids(4, 3)
    rng = np.random.default_rng(0)
    vals = [rng.random((s, 4, 4)) for s in (1, 2, 3, 1, 2)]
    with RegridServer(hbm_budget=10**9, slots=1, backend=be) as srv:
        f0 = srv.submit(gi, go, vals[0], key="g")  # occupies the only slot (blocked in run)
        time.sleep(0.1)
        rest = [srv.submit(gi, go, v, key="g") for v in vals[1:]]  # wait together
        time.sleep(0.1)
        gate.set()
        outs = [f.result(5) for f in [f0, *rest]]
        st = srv.stats()
    m = FakeBackend.matrix("g", 16, 9)
    for v, o in zip(vals, outs):
        np.testing.assert_array_equal(o, v.reshape(v.shape[0], 16) @ m.T)
    assert be.builds == ["g"]
    assert [len(b) for b in be.batches] == [1, 4]  # the four waiting requests went as one apply
    assert st["builds"] == 1 and st["batches"] == 2 and st["done"] == 5


def test_max_batch_stack_splits_batches():
    gate = threading.Event()
    be = FakeBackend(gate=gate)
    gi, go = grids(2, 2)
    with RegridServer(hbm_budget=10**9, slots=1, backend=be, max_batch_stack=4) as srv:
        fs = [srv.submit(gi, go, np.ones((3, 2, 2)), key="k") for _ in range(4)]
        time.sleep(0.1)
        gate.set()
        for f in fs:
            f.result(5)
    assert all(sum(3 for _ in b) <= 4 or len(b) == 1 for b in be.batches)
    assert sum(len(b) for b in be.batches) == 4


def test_admission_respects_budget_and_overlaps():
    be = FakeBackend(run_delay=0.05)
    gi, go = grids(8, 8)
    # each request: 1 x (64 + 64) x 8 B = 1024 B of values; each build
    # 12,800 B of scratch + 32,768 B of weights
    budget = 3 * (1024 + 12800 + 32768)
    with RegridServer(hbm_budget=budget, slots=8, cache_bytes=budget, backend=be) as srv:
        fs = [srv.submit(gi, go, np.ones((1, 8, 8)), key=f"g{k}") for k in range(12)]
        for f in fs:
            f.result(10)
        st = srv.stats()
    assert st["peak_bytes"] <= budget
    assert be.max_active >= 2  # distinct grids ran at the same time
    assert be.max_active <= 3  # but no more than the budget allows
    assert st["evictions"] > 0 and len(be.freed) >= st["evictions"]


def test_oversized_request_fails_alone():
    be = FakeBackend()
    gi, go = grids(8, 8)
    with RegridServer(hbm_budget=5000, slots=2, backend=be) as srv:
        big = srv.submit(gi, go, np.ones((64, 8, 8)), key="big")
        with pytest.raises(MemoryError):
            big.result(5)
        gs, gos = grids(2, 2)
        ok = srv.submit(gs, gos, np.ones((1, 2, 2)), key="small")
        assert ok.result(5).shape == (1, 4)


def test_build_failure_reaches_every_waiting_request():
    be = FakeBackend(fail_build={"bad"})
    gi, go = grids(3, 3)
    with RegridServer(hbm_budget=10**9, slots=2, backend=be) as srv:
        bad = [srv.submit(gi, go, np.ones((1, 3, 3)), key="bad") for _ in range(3)]
        good = srv.submit(gi, go, np.ones((1, 3, 3)), key="good")
        for f in bad:
            with pytest.raises(RuntimeError, match="build failed"):
                f.result(5)
        assert good.result(5).shape == (1, 9)


def test_cancelled_requests_never_run():
    """Fault injection on the host: a client cancels queued requests.  A
    request cancelled before admission is dropped (its future reports
    cancelled, the backend never sees it); the others still run and are
    batched as usual; an admitted request can no longer be cancelled."""
    gate = threading.Event()
    be = FakeBackend(gate=gate)
    gi, go = grids(4, 3)
    with RegridServer(hbm_budget=10**9, slots=1, backend=be) as srv:
        f0 = srv.submit(gi, go, np.ones((1, 4, 4)), key="g")  # holds the only slot
        time.sleep(0.1)
        assert not f0.cancel()  # running
        waiting = [srv.submit(gi, go, np.full((1, 4, 4), k), key="g") for k in range(4)]
        other = srv.submit(gi, go, np.ones((1, 4, 4)), key="h")
        time.sleep(0.05)
        assert waiting[1].cancel() and waiting[3].cancel()
        gate.set()
        f0.result(5)
        kept = [waiting[0].result(5), waiting[2].result(5)]
        other.result(5)
        st = srv.stats()
    assert waiting[1].cancelled() and waiting[3].cancelled()
    m = FakeBackend.matrix("g", 16, 9)
    np.testing.assert_array_equal(kept[1], np.full((1, 16), 2.0) @ m.T)
    assert sum(len(b) for b in be.batches) == 4  # f0, waiting[0], waiting[2], other
    assert st["cancelled"] == 2 and st["done"] == 4


class FlakyAllocBackend(FakeBackend):
    """A backend whose device allocations fail on chosen calls, as
    cudaMallocAsync does when the device is out of memory."""

    def __init__(self, fail_build_calls=(), fail_run_calls=(), **kw):
        super().__init__(**kw)
        self.fail_build_calls, self.fail_run_calls = set(fail_build_calls), set(fail_run_calls)
        self.n_build = self.n_run = 0

    def build(self, slot, req):
        with self.lock:
            self.n_build += 1
            fail = self.n_build in self.fail_build_calls
        if fail:
            raise MemoryError("cudaMallocAsync: out of memory (injected)")
        return super().build(slot, req)

    def run(self, slot, m, reqs):
        with self.lock:
            self.n_run += 1
            fail = self.n_run in self.fail_run_calls
        if fail:
            raise MemoryError("cudaMallocAsync: out of memory (injected)")
        return super().run(slot, m, reqs)


def test_allocation_failures_fail_their_request_alone():
    """Fault injection on the host: an allocation fails inside an admitted
    request's build, and another inside an apply.  Each fails its own
    request with the error; the reserved device footprint is given back (the
    server's accounting returns to the cache alone), the failed grid is
    built again by its next request, and other requests are unaffected."""
    be = FlakyAllocBackend(fail_build_calls={1}, fail_run_calls={2})
    gi, go = grids(4, 3)
    with RegridServer(hbm_budget=10**9, slots=1, backend=be) as srv:
        first = srv.submit(gi, go, np.ones((1, 4, 4)), key="a")  # build 1 fails
        with pytest.raises(MemoryError, match="injected"):
            first.result(5)
        assert srv._transient == 0 and "a" not in srv.cache
        ok = srv.submit(gi, go, np.ones((1, 4, 4)), key="a")  # build 2 succeeds, run 1
        ok.result(5)
        bad_run = srv.submit(gi, go, np.ones((1, 4, 4)), key="a")  # cached, run 2 fails
        with pytest.raises(MemoryError, match="injected"):
            bad_run.result(5)
        again = srv.submit(gi, go, np.ones((1, 4, 4)), key="a")  # run 3
        np.testing.assert_array_equal(again.result(5), np.ones((1, 16)) @ FakeBackend.matrix("a", 16, 9).T)
        with srv._cv:
            assert srv._transient == 0 and srv.cache.used == srv._in_use()
        st = srv.stats()
    assert be.builds == ["a"]  # the failed build never reached the cache; the second one did
    assert st["builds"] == 1 and st["done"] == 4


def test_bad_request_and_close():
    be = FakeBackend(run_delay=0.02)
    gi, go = grids(3, 3)
    srv = RegridServer(hbm_budget=10**9, slots=2, backend=be)
    with pytest.raises(ValueError):
        srv.submit((gi[0][0], gi[1][0]), go, np.ones((1, 3, 3))).result(1)  # 1D grids
    fs = [srv.submit(gi, go, np.ones((1, 3, 3)), key=f"k{i % 3}") for i in range(9)]
    srv.close()  # drains what was queued
    assert all(f.done() and f.exception() is None for f in fs)
    with pytest.raises(RuntimeError, match="closed"):
        srv.submit(gi, go, np.ones((1, 3, 3)), key="x").result(1)
    assert len(be.freed) == len(set(be.builds))  # the cache was emptied


def test_unkeyed_requests_are_hashed_and_batched_by_grid():
    """Requests without a key are keyed by the grids' hash (off the
    submitting thread); equal grids share weights, different grids do not."""
    from regridding_gb300.serving import grid_key

    be = FakeBackend(run_delay=0.01)
    gi, go = grids(4, 3)
    gi2 = (gi[0] + 1e-12, gi[1])
    assert grid_key(gi, go) == grid_key(tuple(a.copy() for a in gi), go)
    assert grid_key(gi, go) != grid_key(gi2, go)
    srv = RegridServer(hbm_budget=10**9, slots=2, backend=be)
    fs = [srv.submit(gi if i % 2 else gi2, go, np.ones((1, 4, 4))) for i in range(10)]
    srv.close()  # waits for the keying pool, then drains
    assert all(f.exception() is None for f in fs)
    assert len(set(be.builds)) == 2 and len(be.builds) == 2


class FakeBatchBackend(FakeBackend):
    def __init__(self, **kw):
        super().__init__(**kw)
        self.build_calls = []

    def build_many(self, slot, reqs):
        with self.lock:
            self.build_calls.append([r.key for r in reqs])
        out = []
        for r in reqs:
            try:
                out.append(self.build(slot, r))
            except Exception as e:  # noqa: BLE001
                out.append(e)
        return out


def test_cobuilds_share_one_batched_build():
    """While a slot is busy, requests for several new grids wait; the next
    job builds all their weights in one batched build, later jobs find them
    cached, and a grid whose build fails fails only its own requests."""
    gate = threading.Event()
    be = FakeBatchBackend(gate=gate, fail_build={"k3"})
    gi, go = grids(3, 2)
    with RegridServer(hbm_budget=10**9, slots=1, backend=be, max_cobuild=8, cobuild_max_cells=100) as srv:
        first = srv.submit(gi, go, np.ones((1, 3, 3)), key="k0")  # holds the slot
        time.sleep(0.1)
        fs = {k: srv.submit(gi, go, np.ones((1, 3, 3)), key=k) for k in ("k1", "k2", "k3", "k4")}
        time.sleep(0.1)
        gate.set()
        first.result(5)
        for k, f in fs.items():
            if k == "k3":
                with pytest.raises(RuntimeError, match="build failed"):
                    f.result(5)
            else:
                np.testing.assert_array_equal(f.result(5), np.ones((1, 9)) @ FakeBackend.matrix(k, 9, 4).T)
        st = srv.stats()
    assert ["k1", "k2", "k3", "k4"] in be.build_calls  # one batched build for the four waiting grids
    assert st["builds"] == 4  # k0, k1, k2, k4


def test_grid_key_memo_follows_the_object():
    """A read-only array is hashed once; a new array that reuses a freed
    one's memory and shape with other contents gets its own key."""
    import gc

    from regridding_gb300.serving import grid_key

    def ro(v):
        a = np.full((5, 5), v)
        a.setflags(write=False)
        return a

    keys = set()
    for v in range(20):
        a, b = ro(v), ro(0.0)
        keys.add(grid_key((a, b), (b, b)))
        del a
        gc.collect()
    assert len(keys) == 20
