"""Served conservative regridding: a request loop over the GPU path.

Requests (an input vertex grid, an output vertex grid and a stack of values)
arrive at any time from any thread.  The server

* keys built weights by a hash of the two grids and keeps them resident on
  the device in an LRU whose bytes count against the HBM budget,
* admits a request when its device footprint (values in and out, plus the
  build scratch when its weights are not cached) fits in the budget next to
  the cache and the requests already running,
* runs admitted work on slots: one worker thread and one CUDA stream each, so
  builds, copies and applies of different requests overlap on the GPU (the
  library releases the GIL inside every call),
* batches continuously: requests for the same grid pair that are waiting when
  a slot frees up go out together as one apply over their concatenated
  stacks, and a request that arrives while others run joins the next batch
  of its grid.

Each result is the same alone and in the mix: a slice of the batched apply is
computed by the same per-row sums as an apply of that request alone.

The upstream has no serving layer; this module is the served form of
``regrid(method="conservative")`` for 2D grids
(regridding/_regrid/_regrid.py:12-149 with
regridding/_weights/_weights_conservative_2d/_weights_conservative_2d.py:76-126).
Like the upstream ``weights()`` for 2D conservative grids, the output
coordinates get the seeded 1e-9 jitter before a build (``perturb=True``,
``seed=42``; regridding/_util.py:121-129), so a served result equals the
upstream's ``regrid()`` of the same request; the cache key covers the
unperturbed grids and the two settings.
"""

from __future__ import annotations

import collections
import ctypes
import sys
import threading
import time
import weakref
from concurrent.futures import Future, ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np

from . import _device, _lib, _util

__all__ = ["RegridServer", "WeightsLRU", "grid_key", "regrid_plain", "GpuBackend"]


# ---------------------------------------------------------------------------
# keys
# ---------------------------------------------------------------------------

_key_memo: dict[tuple, tuple] = {}
_key_memo_lock = threading.Lock()


def _hash_array(a: np.ndarray) -> tuple:
    return _device.content_hash(a)


def _forget(memo: tuple) -> None:
    with _key_memo_lock:
        _key_memo.pop(memo, None)


def grid_key(grid_input, grid_output) -> tuple:
    """Cache key of a grid pair: dtype, shape and two seeded 64-bit hashes of
    every coordinate array.  Read-only arrays are hashed once per object (the
    memo holds a weak reference and is checked against the very object, so a
    new array that reuses a freed one's address is hashed afresh)."""
    parts = []
    for a in (*grid_input, *grid_output):
        a = np.asarray(a)
        if not a.flags.writeable:
            memo = (id(a), a.__array_interface__["data"][0], a.shape)
            with _key_memo_lock:
                hit = _key_memo.get(memo)
            if hit is not None and hit[0]() is a:
                parts.append(hit[1])
                continue
            h = _hash_array(a)
            try:
                ref = weakref.ref(a)
            except TypeError:  # not weak-referenceable: no memo
                parts.append(h)
                continue
            with _key_memo_lock:
                _key_memo[memo] = (ref, h)
            weakref.finalize(a, _forget, memo)
            parts.append(h)
        else:
            parts.append(_hash_array(a))
    return tuple(parts)


# ---------------------------------------------------------------------------
# the device-resident weights cache
# ---------------------------------------------------------------------------


@dataclass
class _Entry:
    weights: object
    nbytes: int
    refs: int = 0


class WeightsLRU:
    """Built weights by key, least recently used first.

    Every entry's device bytes are counted; entries that a running job holds
    (``refs > 0``) are never evicted.  Not thread-safe by itself: the server
    calls it under its own lock.
    """

    def __init__(self, capacity_bytes: int, free=None):
        self.capacity = int(capacity_bytes)
        self.used = 0
        self._d: collections.OrderedDict = collections.OrderedDict()
        self._free = free or (lambda w: None)
        self.hits = 0
        self.misses = 0
        self.evictions = 0

    def __contains__(self, key) -> bool:
        return key in self._d

    def __len__(self) -> int:
        return len(self._d)

    def keys(self) -> list:
        return list(self._d)

    def acquire(self, key):
        """The weights of key with a reference taken, or None."""
        e = self._d.get(key)
        if e is None:
            self.misses += 1
            return None
        self.hits += 1
        self._d.move_to_end(key)
        e.refs += 1
        return e.weights

    def insert(self, key, weights, nbytes: int):
        """Add weights with one reference taken (by the inserting job)."""
        old = self._d.pop(key, None)
        if old is not None:
            self.used -= old.nbytes
            self._free(old.weights)
        self._d[key] = _Entry(weights, int(nbytes), 1)
        self.used += int(nbytes)
        self._trim(self.capacity)

    def release(self, key) -> None:
        e = self._d.get(key)
        if e is not None and e.refs > 0:
            e.refs -= 1
        self._trim(self.capacity)

    def evictable(self) -> int:
        return sum(e.nbytes for e in self._d.values() if e.refs == 0)

    def shrink_by(self, nbytes: int) -> None:
        """Evict unreferenced entries, oldest first, until nbytes are freed
        (or nothing evictable is left)."""
        self._trim(self.used - nbytes)

    def _trim(self, limit: int) -> None:
        if self.used <= limit:
            return
        for key in list(self._d):
            if self.used <= limit:
                break
            e = self._d[key]
            if e.refs == 0:
                del self._d[key]
                self.used -= e.nbytes
                self.evictions += 1
                self._free(e.weights)

    def clear(self) -> None:
        for e in self._d.values():
            self._free(e.weights)
        self._d.clear()
        self.used = 0


# ---------------------------------------------------------------------------
# requests and the GPU backend
# ---------------------------------------------------------------------------


@dataclass(eq=False)
class _Request:
    grid_input: tuple
    grid_output: tuple
    values: object  # host tensor (stack, n_in) float32/float64
    out: object  # host tensor (stack, n_out)
    stack: int
    n_in: int
    n_out: int
    key: tuple
    future: Future
    t_arrival: float
    result: object = None
    grids_hashed: bool = False  # key = grid_key(grids) + (perturb, seed)
    t_start: float = 0.0  # its job started on a slot
    t_built: float = 0.0  # its weights were ready (build jobs)
    t_done: float = 0.0
    batch: int = 0


@dataclass(eq=False)
class _Job:
    key: tuple
    requests: list
    build: bool
    footprint: int
    weights: object = None
    slot: int = -1
    t_start: float = 0.0
    cobuild: list = None  # one waiting request per other grid built in the same batched build


class GpuBackend:
    """Builds and applies through ``libregrid_gb300.so`` on the slots' streams."""

    # device bytes per (input + output) cell of a build: raw triples, the
    # bucket sort's keys and permutation, and the CSR (measured on the
    # 2048^2 -> 1536^2 build: about 220 B per cell)
    BUILD_BYTES_PER_CELL = 256

    def __init__(self, accumulate: str = "fast", perturb: bool = True, seed: int = 42, disk_cache=None,
                 urgent_builds: bool = False):
        self.torch = _device.torch()
        self.accumulate = accumulate
        self.urgent_builds = urgent_builds
        self.perturb = perturb
        self.seed = seed
        # weights files shared with store.WeightsDiskCache.weights(..., method="conservative")
        self.disk = disk_cache
        self.disk_loads = 0
        self._disk_stream = self.torch.cuda.Stream() if disk_cache is not None else None
        self._writer = ThreadPoolExecutor(max_workers=1, thread_name_prefix="regrid-disk") \
            if disk_cache is not None else None

    def grids(self, grid_input, grid_output):
        """The coordinates a build sees: the output jittered as the upstream
        ``weights(method="conservative")`` does by default."""
        if not self.perturb:
            return grid_input, grid_output
        gi, go, *_ = _util.normalize_input_output_coordinates(grid_input, grid_output, None, None,
                                                               perturb=True, seed=self.seed)
        return gi, go

    class Slot:
        """A slot's compute stream and the stream its input copies use; with
        ``urgent`` also a high-priority stream for the jobs that build (the
        work on the critical path of the slowest requests)."""

        def __init__(self, torch, urgent: bool = False):
            self.stream = torch.cuda.Stream()
            self.copy = torch.cuda.Stream()
            self.urgent = None
            if urgent:
                view = GpuBackend.Slot.__new__(GpuBackend.Slot)
                view.stream = torch.cuda.Stream(priority=-1)
                view.copy = self.copy
                view.urgent = None
                self.urgent = view

    def make_slot(self, index: int):
        return GpuBackend.Slot(self.torch, self.urgent_builds)

    def stage(self, slot, requests: list):
        """Start copying the requests' stacks to one device buffer on the
        slot's copy stream (so that they travel while the weights build);
        returns the buffer and the event that marks the copies' end."""
        t = self.torch
        vdt = requests[0].values.dtype
        if not all(r.values.dtype == vdt for r in requests):
            vdt = t.float64
        n_in = requests[0].n_in
        with t.cuda.stream(slot.copy):
            vin = t.empty((sum(r.stack for r in requests), n_in), dtype=vdt, device="cuda")
            off = 0
            for r in requests:
                vin[off:off + r.stack].copy_(r.values, non_blocking=True)
                off += r.stack
            done = t.cuda.Event()
            done.record(slot.copy)
        return vin, done

    def prepare(self, values, out, n_in: int, n_out: int):
        """Host tensors for a request: values viewed as (stack, n_in); out
        (given or newly allocated) as (stack, n_out)."""
        t = self.torch
        v = values if isinstance(values, t.Tensor) else t.from_numpy(np.ascontiguousarray(values))
        if v.dtype not in (t.float32, t.float64):
            v = v.to(t.float64)
        v = v.reshape(-1, n_in)
        odt = t.float32 if (self.accumulate == "fast" and v.dtype == t.float32) else t.float64
        if out is None:
            o = t.empty((v.shape[0], n_out), dtype=odt)
        else:
            o = out if isinstance(out, t.Tensor) else t.from_numpy(out)
            if o.dtype != odt:
                raise ValueError(f"out must be {odt}, got {o.dtype}")
            o = o.reshape(v.shape[0], n_out)
        return v, o

    def request_bytes(self, req: _Request) -> int:
        return req.stack * (req.n_in * req.values.element_size() + req.n_out * req.out.element_size())

    def build_bytes(self, req: _Request) -> int:
        return self.BUILD_BYTES_PER_CELL * (req.n_in + req.n_out)

    def disk_key(self, req: _Request) -> str | None:
        """Name of the request's weights in the disk cache: the grid hashes
        of its serving key, with the build's perturbation and seed."""
        from . import store

        grids = req.key[:-2] if req.grids_hashed else None
        return store.weights_key(tuple(req.grid_input), tuple(req.grid_output), method="conservative",
                                 perturb=self.perturb, seed=self.seed, grids=grids)

    def _footprint(self, dw) -> int:
        nbytes = ctypes.c_int64()
        _lib.call("rg_weights_device_bytes", dw.handle, ctypes.byref(nbytes))
        # room for the float32 weights and tile lists the first apply makes
        return nbytes.value + dw.nnz * 6 + (dw.n_out // 32 + 1) * 16

    def _range(self, name: str):
        """An NVTX range on the host timeline (Nsight tools)."""
        return self.torch.cuda.nvtx.range(name)

    def build(self, slot, req: _Request):
        with self._range("serve.build"):
            return self._build(slot, req)

    def _build(self, slot, req: _Request):
        dkey = self.disk_key(req) if self.disk is not None else None
        if dkey is not None:
            stored = self.disk.get(dkey)
            if stored is not None:
                ii, oo, vv = stored[0].reshape(-1)[0]
                xi, xo = req.grid_input[0], req.grid_output[0]
                with self.torch.cuda.stream(slot.stream):
                    dw = _device.DeviceWeights.from_coo(ii, oo, vv, req.n_in, req.n_out,
                                                        (xo.shape[0] - 1, xo.shape[1] - 1),
                                                        (xi.shape[0] - 1, xi.shape[1] - 1))
                self.disk_loads += 1
                return dw, self._footprint(dw)
        gi, go = self.grids(req.grid_input, req.grid_output)
        with self.torch.cuda.stream(slot.stream):
            dw = _device.build_conservative_2d(gi, go)
        if dkey is not None:
            self._persist(slot, dkey, dw, np.shape(req.grid_input[0]), np.shape(req.grid_output[0]))
        return dw, self._footprint(dw)

    def _persist(self, slot, key: str, dw, shape_in, shape_out) -> None:
        """Export the new weights on the slot's stream, copy them to pinned
        host memory on a side stream, and write the file from the writer
        thread once the copy is done (the slot goes on meanwhile)."""
        t = self.torch
        with t.cuda.stream(slot.stream):
            dev = dw.export()
            exported = t.cuda.Event()
            exported.record(slot.stream)
        side = self._disk_stream
        side.wait_event(exported)
        with t.cuda.stream(side):
            host = []
            for d in dev:
                d.record_stream(side)
                h = t.empty(d.shape, dtype=d.dtype, pin_memory=True)
                h.copy_(d, non_blocking=True)
                host.append(h)
            copied = t.cuda.Event()
            copied.record(side)

        def write():
            copied.synchronize()
            array = np.empty((), dtype=object)
            array[()] = tuple(h.numpy() for h in host)
            self.disk.put(key, (array, tuple(shape_in), tuple(shape_out)), {"method": "conservative"})
            del dev[:]

        self._writer.submit(write)

    def flush(self) -> None:
        """Wait for the weights files still being written."""
        if self._writer is not None:
            self._writer.submit(lambda: None).result()

    def build_many(self, slot, reqs: list) -> list:
        """Weights of several grid pairs in one batched build: per request
        (weights, device bytes) or the exception of its failed build."""
        pairs = [self.grids(r.grid_input, r.grid_output) for r in reqs]
        with self.torch.cuda.stream(slot.stream):
            built = _device.build_conservative_2d_batch(pairs)
        out = []
        for dw in built:
            if isinstance(dw, Exception):
                out.append(dw)
                continue
            nbytes = ctypes.c_int64()
            _lib.call("rg_weights_device_bytes", dw.handle, ctypes.byref(nbytes))
            out.append((dw, nbytes.value + dw.nnz * 6 + (dw.n_out // 32 + 1) * 16))
        return out

    def run(self, slot, weights, requests: list, staged=None) -> None:
        with self._range("serve.apply"):
            self._run(slot, weights, requests, staged)

    # a request whose stack in host memory is at least this large is applied
    # by rg_apply_host: chunks of ~128 MB are copied in, applied and copied
    # out on three streams, so the two copy directions and the kernels overlap
    PIPELINE_BYTES = 192 << 20

    def _pipelined(self, requests: list, staged) -> bool:
        if staged is not None or len(requests) != 1:
            return False
        r = requests[0]
        v, o = r.values, r.out
        return (v.device.type == "cpu" and o.device.type == "cpu" and v.is_contiguous() and o.is_contiguous()
                and v.is_pinned() and o.is_pinned() and v.numel() * v.element_size() >= self.PIPELINE_BYTES)

    def _run(self, slot, weights, requests: list, staged=None) -> None:
        t = self.torch
        if self._pipelined(requests, staged):
            r = requests[0]
            dt = {t.float32: _lib.RG_F32, t.float64: _lib.RG_F64}
            _lib.call("rg_apply_host", weights.handle, ctypes.c_void_p(r.values.data_ptr()), dt[r.values.dtype],
                      ctypes.c_void_p(r.out.data_ptr()), dt[r.out.dtype], int(r.stack), _lib.RG_ACC[self.accumulate],
                      0, ctypes.c_void_p(slot.stream.cuda_stream))
            slot.stream.synchronize()
            return
        with t.cuda.stream(slot.stream):
            if staged is not None:
                vin, done = staged
                slot.stream.wait_event(done)
                vin.record_stream(slot.stream)  # used on this stream too (allocator bookkeeping)
            else:
                vdt = requests[0].values.dtype
                if not all(r.values.dtype == vdt for r in requests):
                    vdt = t.float64
                vin = t.empty((sum(r.stack for r in requests), weights.n_in), dtype=vdt, device="cuda")
                off = 0
                for r in requests:
                    vin[off:off + r.stack].copy_(r.values, non_blocking=True)
                    off += r.stack
            total = vin.shape[0]
            odt = requests[0].out.dtype
            out = weights.apply(vin, out=t.empty((total, weights.n_out), dtype=odt, device="cuda"),
                                accumulate=self.accumulate)
            off = 0
            for r in requests:
                r.out.copy_(out[off:off + r.stack], non_blocking=True)
                off += r.stack
            slot.stream.synchronize()

    def free(self, weights) -> None:
        weights.free()


# ---------------------------------------------------------------------------
# the server
# ---------------------------------------------------------------------------


class RegridServer:
    """Continuous-batching request loop for 2D conservative regridding.

    Parameters
    ----------
    hbm_budget:
        Device bytes the server may hold at once: cached weights plus the
        footprints of running requests (80 GB by default).
    slots:
        Worker threads, each with its own CUDA stream.
    cache_bytes:
        Upper bound of the weights cache (default: half the budget).
    max_batch_stack:
        Largest concatenated stack of one batched apply.
    accumulate:
        ``"fast"`` (float32 stacks give float32 results, FMA accumulation) or
        ``"exact"`` (float64 results bit-identical to the upstream apply).
    perturb, seed:
        The upstream's default output-coordinate jitter before a build.
    intake_threads:
        Threads that hash the grids of requests submitted without a key.
    max_cobuild, cobuild_max_cells:
        A job that builds the weights of a small grid pair (at most
        ``cobuild_max_cells`` input cells) also builds those of up to
        ``max_cobuild`` other small waiting pairs in the same batched build
        (their requests then find the weights cached).  Small builds are
        dominated by fixed per-build costs that a batch pays once; large
        builds gain little and would make the small ones wait.
    urgent_builds:
        Run the jobs that build on high-priority CUDA streams, so that the
        block scheduler serves them before the applies of resident grids.
    switch_interval:
        If given, ``sys.setswitchinterval`` for the process: how long a
        thread may hold the GIL before another runnable thread gets it.
    disk_cache:
        A :class:`~regridding_gb300.store.WeightsDiskCache`: a build first
        looks for the weights file of its grid pair there (an upload instead
        of a build), and new weights are written to it in the background.
        The files are those of ``disk_cache.weights(grid_input, grid_output,
        method="conservative")``, so servers and batch jobs share them.
    """

    def __init__(self, hbm_budget: float = 80e9, slots: int = 4, cache_bytes: float | None = None,
                 max_batch_stack: int = 64, accumulate: str = "fast", perturb: bool = True, seed: int = 42,
                 intake_threads: int = 4, max_cobuild: int = 0, cobuild_max_cells: int = 512 * 512,
                 backend=None, disk_cache=None, urgent_builds: bool = False,
                 switch_interval: float | None = None):
        if accumulate not in ("fast", "exact"):
            raise ValueError(f"accumulate must be 'fast' or 'exact', got {accumulate!r}")
        if switch_interval is not None:
            # the interpreter's thread switch interval bounds how long a slot
            # thread back from a native call waits for the GIL (process-wide)
            sys.setswitchinterval(switch_interval)
        self.backend = backend if backend is not None else GpuBackend(accumulate, perturb, seed, disk_cache,
                                                                      urgent_builds)
        self._key_extra = (bool(perturb), int(seed))
        self.budget = int(hbm_budget)
        self.cache = WeightsLRU(int(cache_bytes if cache_bytes is not None else hbm_budget // 2),
                                free=self.backend.free)
        self.max_batch_stack = int(max_batch_stack)
        self.max_cobuild = int(max_cobuild) if hasattr(self.backend, "build_many") else 0
        self.cobuild_max_cells = int(cobuild_max_cells)
        # one lock; the scheduler waits on _cv, each slot's worker on its own
        # condition, so that a state change wakes only the thread it concerns
        # (waking all 17 threads on every change cost host time under load)
        lock = threading.RLock()
        self._cv = threading.Condition(lock)
        self._slot_cv = [threading.Condition(lock) for _ in range(slots)]
        self._pending: collections.deque[_Request] = collections.deque()
        self._building: set = set()
        self._transient = 0  # footprints of admitted jobs
        self.peak_bytes = 0
        self._free_slots = list(range(slots))
        self._slot_streams = [self.backend.make_slot(i) for i in range(slots)]
        self._slot_jobs: list[_Job | None] = [None] * slots
        self._running = True
        self._intake = ThreadPoolExecutor(max_workers=intake_threads, thread_name_prefix="regrid-intake")
        self._intake_n = 0  # requests being keyed
        self.n_batches = 0
        self.n_builds = 0
        self.n_done = 0
        self.n_cancelled = 0
        self._workers = [threading.Thread(target=self._worker, args=(i,), daemon=True, name=f"regrid-slot-{i}")
                         for i in range(slots)]
        for w in self._workers:
            w.start()
        self._scheduler = threading.Thread(target=self._schedule, daemon=True, name="regrid-scheduler")
        self._scheduler.start()

    # -- public -------------------------------------------------------------

    def submit(self, grid_input, grid_output, values, out=None, key=None, t_arrival: float | None = None) -> Future:
        """Queue one regrid; the future's result is the output stack
        (values' leading axes, then the output cells flattened row-major)."""
        fut: Future = Future()
        try:
            gi = tuple(np.asarray(a) for a in grid_input)
            go = tuple(np.asarray(a) for a in grid_output)
            if len(gi) != 2 or len(go) != 2 or gi[0].ndim != 2 or go[0].ndim != 2:
                raise ValueError("the served form regrids 2D vertex grids (x, y)")
            n_in = (gi[0].shape[0] - 1) * (gi[0].shape[1] - 1)
            n_out = (go[0].shape[0] - 1) * (go[0].shape[1] - 1)
            v, o = self.backend.prepare(values, out, n_in, n_out)
            req = _Request(gi, go, v, o, int(v.shape[0]), n_in, n_out, key, fut,
                           time.perf_counter() if t_arrival is None else t_arrival)
        except Exception as e:  # bad request: fail its future, keep serving
            fut.set_exception(e)
            return fut
        fut.request = req  # timing fields for callers that measure latency
        with self._cv:
            if not self._running:
                fut.set_exception(RuntimeError("server is closed"))
                return fut
            if key is not None:
                self._pending.append(req)
                self._cv.notify()
                return fut
            self._intake_n += 1
        # hashing the grids (native, GIL released) runs on the intake pool so
        # that a client submitting many requests is not held up by it
        self._intake.submit(self._key_and_queue, req)
        return fut

    def _key_and_queue(self, req: _Request) -> None:
        try:
            req.key = grid_key(req.grid_input, req.grid_output) + self._key_extra
            req.grids_hashed = True
        except Exception as e:  # noqa: BLE001
            req.future.set_exception(e)
            with self._cv:
                self._intake_n -= 1
                self._cv.notify()
            return
        with self._cv:
            self._intake_n -= 1
            self._pending.append(req)
            self._cv.notify()

    def close(self, wait: bool = True) -> None:
        """Stop accepting requests; finish what is queued when wait, else fail it."""
        with self._cv:
            accepting = self._running
            self._running = False  # no new submissions
        if accepting:
            self._intake.shutdown(wait=True)  # requests being keyed reach the queue
        with self._cv:
            if not wait:
                while self._pending:
                    self._pending.popleft().future.set_exception(RuntimeError("server closed"))
            self._running = False
            self._wake_all()
        self._scheduler.join()
        with self._cv:
            self._wake_all()
        for w in self._workers:
            w.join()
        with self._cv:
            self.cache.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def stats(self) -> dict:
        with self._cv:
            return {"done": self.n_done, "batches": self.n_batches, "builds": self.n_builds,
                    "cancelled": self.n_cancelled,
                    "cache_entries": len(self.cache), "cache_bytes": self.cache.used,
                    "cache_hits": self.cache.hits, "cache_misses": self.cache.misses,
                    "evictions": self.cache.evictions, "peak_bytes": self.peak_bytes, "budget": self.budget}

    # -- scheduling ---------------------------------------------------------

    def _in_use(self) -> int:
        return self.cache.used + self._transient

    def _schedule(self) -> None:
        with self._cv:
            while True:
                try:
                    progressed = self._dispatch()
                except Exception as e:  # noqa: BLE001 - a scheduling bug must not stall the queue
                    progressed = True
                    while self._pending:
                        self._pending.popleft().future.set_exception(e)
                if not self._running and not self._pending and not self._intake_n:
                    break
                if not progressed:
                    self._cv.wait(timeout=0.05)
            # let the workers finish and exit
            self._wake_all()

    def _wake_all(self) -> None:
        """Wake the scheduler and every slot (lock held)."""
        self._cv.notify_all()
        for cv in self._slot_cv:
            cv.notify_all()

    def _dispatch(self) -> bool:
        """Admit as many waiting requests as slots and memory allow (lock held)."""
        progressed = False
        while self._free_slots and self._pending:
            job = self._next_job()
            if job is None:
                break
            slot = self._free_slots.pop(0)
            job.slot = slot
            self._slot_jobs[slot] = job
            self._transient += job.footprint
            self.peak_bytes = max(self.peak_bytes, self._in_use())
            self.n_batches += 1
            if job.build:
                self._building.add(job.key)
                for r in job.cobuild or ():
                    self._building.add(r.key)
            progressed = True
            self._slot_cv[slot].notify()
        return progressed

    def _drop_cancelled(self) -> None:
        """Forget waiting requests whose futures the client cancelled."""
        n = sum(1 for r in self._pending if r.future.cancelled())
        if n:
            self._pending = collections.deque(r for r in self._pending if not r.future.cancelled())
            self.n_cancelled += n

    def _next_job(self) -> _Job | None:
        """The oldest waiting request whose grid is not being built, with the
        other waiting requests of its grid, if its footprint fits; None when
        the oldest admissible request must wait for memory.  A request
        cancelled by its client before admission is dropped; once admitted
        it runs to the end (its future can no longer be cancelled)."""
        self._drop_cancelled()
        for head in list(self._pending):
            if head.key in self._building:
                continue  # its weights are on the way; later requests may go first
            group, stack = [], 0
            for r in self._pending:
                if r.key == head.key and (not group or stack + r.stack <= self.max_batch_stack):
                    group.append(r)
                    stack += r.stack
            cached = head.key in self.cache
            footprint = sum(self.backend.request_bytes(r) for r in group)
            if not cached:
                footprint += self.backend.build_bytes(head)
            if footprint > self.budget:
                if len(group) > 1:
                    group = [head]
                    footprint = self.backend.request_bytes(head) + (0 if cached else self.backend.build_bytes(head))
                if footprint > self.budget:
                    self._pending.remove(head)
                    head.future.set_exception(MemoryError(
                        f"request needs {footprint} device bytes, more than the budget of {self.budget}"))
                    return self._next_job() if self._pending else None
            excess = self._in_use() + footprint - self.budget
            if excess > 0:
                # evict unreferenced weights, oldest first, until the job fits
                self.cache.shrink_by(excess)
                if self._in_use() + footprint > self.budget:
                    return None  # wait for running jobs to free memory (no skipping ahead)
            for r in group:
                self._pending.remove(r)
            # from here on the requests run: a cancel that won the race drops its request
            group = [r for r in group if r.future.set_running_or_notify_cancel()]
            if not group:
                return self._next_job() if self._pending else None
            if group[0] is not head:
                head = group[0]
                footprint = sum(self.backend.request_bytes(r) for r in group) + \
                    (0 if cached else self.backend.build_bytes(head))
            weights = self.cache.acquire(head.key) if cached else None
            if not cached:
                self.cache.misses += 1
            job = _Job(head.key, group, not cached, footprint, weights)
            if not cached and self.max_cobuild > 0 and head.n_in <= self.cobuild_max_cells:
                # other small grids waiting for weights go into the same batched build
                seen = {head.key}
                job.cobuild = []
                for r in self._pending:
                    if len(job.cobuild) >= self.max_cobuild:
                        break
                    if r.key in seen or r.key in self.cache or r.key in self._building:
                        continue
                    if r.n_in > self.cobuild_max_cells:
                        continue
                    extra = self.backend.build_bytes(r)
                    if self._in_use() + job.footprint + extra > self.budget:
                        break
                    seen.add(r.key)
                    job.cobuild.append(r)
                    job.footprint += extra
            return job
        return None

    # -- slots --------------------------------------------------------------

    def _worker(self, slot: int) -> None:
        stream = self._slot_streams[slot]
        while True:
            with self._cv:
                while self._slot_jobs[slot] is None:
                    if not self._running and not self._pending and not self._intake_n:
                        return
                    self._slot_cv[slot].wait(timeout=0.05)
                job = self._slot_jobs[slot]
            self._run(slot, stream, job)

    def _run(self, slot: int, stream, job: _Job) -> None:
        job.t_start = time.perf_counter()
        if job.build and getattr(stream, "urgent", None) is not None:
            stream = stream.urgent
        err = None
        built = False
        cobuild = job.cobuild or []
        staged = None
        t_built = job.t_start
        try:
            if job.build and hasattr(self.backend, "stage"):
                # the stacks travel to the device while the weights build
                staged = self.backend.stage(stream, job.requests)
            if job.build:
                if cobuild:
                    results = self.backend.build_many(stream, [job.requests[0]] + cobuild)
                else:
                    results = [self.backend.build(stream, job.requests[0])]
                with self._cv:
                    for req, res in zip([job.requests[0]] + cobuild, results):
                        head = req is job.requests[0]
                        self._building.discard(req.key)
                        if isinstance(res, Exception):
                            if not head:
                                # the requests of a grid whose build failed fail with it
                                for r in [r for r in self._pending if r.key == req.key]:
                                    self._pending.remove(r)
                                    r.future.set_exception(res)
                            continue
                        self.cache.insert(req.key, res[0], res[1])
                        if not head:
                            self.cache.release(req.key)  # no job holds it yet
                        # the build scratch is returned; the weights now count in the cache
                        scratch = self.backend.build_bytes(req)
                        self._transient -= scratch
                        job.footprint -= scratch
                        self.n_builds += 1
                    self.peak_bytes = max(self.peak_bytes, self._in_use())
                    self._cv.notify_all()
                if isinstance(results[0], Exception):
                    raise results[0]
                job.weights = results[0][0]
                built = True
            t_built = time.perf_counter()
            if staged is not None:
                self.backend.run(stream, job.weights, job.requests, staged)
            else:
                self.backend.run(stream, job.weights, job.requests)
        except Exception as e:  # noqa: BLE001 - reported through the futures
            err = e
        t_done = time.perf_counter()
        with self._cv:
            if job.build and not built:
                self._building.discard(job.key)
                for r in cobuild:
                    self._building.discard(r.key)
            if job.weights is not None or built:
                self.cache.release(job.key)
            self._transient -= job.footprint
            self._slot_jobs[slot] = None
            self._free_slots.append(slot)
            self.n_done += len(job.requests)
            self._cv.notify_all()
        for r in job.requests:
            r.t_start = job.t_start
            r.t_built = t_built if err is None or built else job.t_start
            r.t_done = t_done
            r.batch = len(job.requests)
            if err is not None:
                r.future.set_exception(err)
            else:
                r.future.set_result(r.out)


# ---------------------------------------------------------------------------
# the plain path: one call at a time
# ---------------------------------------------------------------------------


def regrid_plain(grid_input, grid_output, values, accumulate: str = "fast", out=None, perturb: bool = True,
                 seed: int = 42):
    """One request through the library, one call at a time: jitter the
    output grid as ``weights()`` does, upload the grids, build the weights,
    copy the values in, apply, copy the result out and free the weights.  The
    baseline the served form is measured against, and its reference for "the
    same alone"."""
    t = _device.torch()
    backend = GpuBackend(accumulate, perturb, seed)
    gi = tuple(np.asarray(a) for a in grid_input)
    go = tuple(np.asarray(a) for a in grid_output)
    n_in = (gi[0].shape[0] - 1) * (gi[0].shape[1] - 1)
    n_out = (go[0].shape[0] - 1) * (go[0].shape[1] - 1)
    v, o = backend.prepare(values, out, n_in, n_out)
    slot = GpuBackend.Slot.__new__(GpuBackend.Slot)
    slot.stream = slot.copy = t.cuda.current_stream()  # one call at a time: everything in order
    dw = _device.build_conservative_2d(*backend.grids(gi, go))
    try:
        req = _Request(gi, go, v, o, int(v.shape[0]), n_in, n_out, (), Future(), 0.0)
        backend.run(slot, dw, [req])
    finally:
        dw.free()
    return o
