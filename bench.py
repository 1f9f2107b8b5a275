"""Benchmark of the regridding hot path on the 2048^2 -> 1536^2 workload.

One step is one apply of saved conservative weights to a 64-deep float32
stack (64 x 2048 x 2048 -> 64 x 1536 x 1536), the operation a user repeats
for every array regridded between the same two grids.  ``value`` is the
apply's algorithmic HBM traffic divided by its time (inputs resident in HBM;
the 1.07 GB input stack is 8x the L2, so no flush is needed between steps).
The same line reports the weight build (cells/s), the 2D find_indices over
the output vertices, the exact float64-output apply, the end-to-end apply
through the C ABI from host memory, and the CPU baseline (the C restatement
of the upstream loops on every host core).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With N > 1 (torchrun, one process per GPU) every rank runs an independent
replica of the workload; ``value`` sums the ranks' bytes over the slowest
rank's time.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "build cells/s; apply HBM GB/s; served req/s + p50/p99 vs plain GPU path"
STACK = 64
N_IN = 2049
N_OUT = 1537
SERVE_RATE = 500.0
PEAK_FALLBACK_GBS = 6800.0


# ---------------------------------------------------------------------------
# workload bytes
# ---------------------------------------------------------------------------


def apply_bytes(stack: int, n_in: int, n_out: int, nnz: int, b_in: int = 4, b_out: int = 4,
                b_val: int = 4) -> int:
    """Algorithmic bytes of one apply: every input value read once, every
    output written once, the CSR (int32 column + value per entry, int64 row
    pointers) read once."""
    return stack * (n_in * b_in + n_out * b_out) + nnz * (4 + b_val) + (n_out + 1) * 8


# ---------------------------------------------------------------------------
# distributed helpers (replicas: no collective on the data path)
# ---------------------------------------------------------------------------


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def aggregate_seconds(local_seconds: float, world: int, device=None) -> float:
    """Max of the per-rank timings (every rank must call this)."""
    if world <= 1:
        return local_seconds
    import torch
    import torch.distributed as dist

    t = torch.tensor([local_seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------


class ClockSampler:
    """nvidia-smi sampled every 50 ms while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,utilization.gpu,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            time.sleep(0.3)
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self) -> dict:
        rows = []
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) != 9:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), float(parts[2]), float(parts[3]), parts[4:]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        load = [r for r in rows if r[3] >= 50] or rows
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[k] for r in load for k in range(4) if r[4][k + 1].lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in load), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(load), "power_w_max": max(r[2] for r in rows)}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return PEAK_FALLBACK_GBS, "fallback"


def profiled_traffic(kernel: str):
    """DRAM bytes per launch recorded from an ncu capture in profiles/."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(kernel)
    except (OSError, ValueError):
        return None


def time_launches(fn, steps: int, warmup: int, stream, torch):
    """Run fn() warmup + steps times; per-launch CUDA-event durations of the
    timed launches (seconds) and the wall of the whole timed region."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for a, b in ev:
        a.record(stream)
        fn()
        b.record(stream)
    end.record(stream)
    torch.cuda.synchronize()
    per = [a.elapsed_time(b) / 1e3 for a, b in ev]
    return per, start.elapsed_time(end) / 1e3


def run_quick(args, local):
    """Build + fast apply only, at a chosen size: the command profiled by ncu."""
    import torch

    import regridding_gb300 as rg
    from regridding_gb300 import workloads

    torch.cuda.set_device(local)
    gi, go = workloads.cfg2_grids(args.n_in, args.n_out)
    gop = workloads.perturb(go)
    dw = rg.build_conservative_2d(gi, gop)
    values = workloads.cfg2_values_torch(args.stack, args.n_in - 1)
    res = {"quick": True, "n_in": args.n_in, "n_out": args.n_out, "stack": args.stack, "nnz": dw.nnz}
    for mode in args.quick_modes.split(","):
        wide = mode != "fast"
        out = torch.empty((args.stack, (args.n_out - 1) ** 2), dtype=torch.float64 if wide else torch.float32,
                          device="cuda")
        per, wall = time_launches(lambda: dw.apply(values, out=out, accumulate=mode), args.steps, args.warmup,
                                  torch.cuda.current_stream(), torch)
        b = apply_bytes(args.stack, (args.n_in - 1) ** 2, (args.n_out - 1) ** 2, dw.nnz, b_out=8 if wide else 4,
                        b_val=8 if wide else 4)
        res[mode] = {"bytes_per_launch": b, "kernel_ms": round(statistics.mean(per) * 1e3, 4),
                     "GB_per_s": round(b / statistics.mean(per) / 1e9, 1)}
    print(json.dumps(res), flush=True)


def run_serving(args, torch):
    """The served stream (Poisson arrivals at SERVE_RATE req/s, grid sides
    log-uniform in [128, 2048] cells, 70 % of requests on 32 resident grids,
    30 % bringing a new grid, stacks of 1, 8 or 64 float32 slices, 80 GB HBM
    budget) through RegridServer, against the plain path that serves the same
    requests one call at a time."""
    import oracle
    from regridding_gb300 import workloads
    from regridding_gb300.serving import RegridServer, regrid_plain

    n_req = args.serve_requests
    t_gen = time.perf_counter()
    cached, reqs = workloads.served_stream(n_req, rate=SERVE_RATE)
    t_gen = time.perf_counter() - t_gen
    cells = lambda g: (g[0].shape[0] - 1) * (g[0].shape[1] - 1)
    max_in = max(cells(r["pair"][0]) * r["stack"] for r in reqs)
    max_out = max(cells(r["pair"][1]) * r["stack"] for r in reqs)
    rng = np.random.default_rng(7)
    pool = torch.empty(max_in, dtype=torch.float32, pin_memory=True)
    pool.copy_(torch.from_numpy(rng.lognormal(3, 1, max_in).astype(np.float32)))
    sinks = [torch.empty(max_out, dtype=torch.float32, pin_memory=True) for _ in range(4)]

    def values(r):
        return pool[:cells(r["pair"][0]) * r["stack"]].view(r["stack"], -1)

    def sink(i, r):
        return sinks[i % len(sinks)][:cells(r["pair"][1]) * r["stack"]].view(r["stack"], -1)

    def percentiles(lat):
        lat = np.sort(np.asarray(lat)) * 1e3
        return round(float(np.percentile(lat, 50)), 3), round(float(np.percentile(lat, 99)), 3)

    out = {"requests": n_req, "offered_rate": SERVE_RATE, "stream_generation_s": round(t_gen, 2),
           "slots": args.serve_slots,
           "grids": "clients send output grids that already carry their 1e-9 jitter; server and plain path "
                    "both run with perturb=False"}
    for mode in ("poisson", "saturated"):
        # a fresh server per pass: the 32 resident grids are built before the
        # stream starts, every new grid of the stream is built during it
        with RegridServer(hbm_budget=80e9, slots=args.serve_slots, max_batch_stack=64, perturb=False,
                          max_cobuild=args.serve_cobuild, urgent_builds=args.serve_urgent,
                          switch_interval=args.serve_switch_ms / 1e3 if args.serve_switch_ms else None) as srv:
            warm = [srv.submit(gi, go, np.zeros((1, cells(gi)), np.float32)) for gi, go in cached]
            for f in warm:
                f.result()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            futs = []
            for i, r in enumerate(reqs):
                t_arr = t0 + (r["t"] if mode == "poisson" else 0.0)
                if mode == "poisson":
                    delay = t_arr - time.perf_counter()
                    if delay > 0:
                        time.sleep(delay)
                futs.append(srv.submit(*r["pair"], values(r), out=sink(i, r), t_arrival=t_arr))
            for f in futs:
                f.result()
            t_end = max(f.request.t_done for f in futs)
            lat = [f.request.t_done - f.request.t_arrival for f in futs]
            p50, p99 = percentiles(lat)
            new = [f.request.t_done - f.request.t_arrival for f, r in zip(futs, reqs) if r["cached"] < 0]
            old = [f.request.t_done - f.request.t_arrival for f, r in zip(futs, reqs) if r["cached"] >= 0]
            nq = [f.request for f, r in zip(futs, reqs) if r["cached"] < 0]
            out[mode] = {"req_per_s": round(n_req / (t_end - t0), 1), "p50_ms": p50, "p99_ms": p99,
                         "p50_p99_ms_resident_grid": percentiles(old), "p50_p99_ms_new_grid": percentiles(new),
                         "new_grid_p50_p99_ms": {"wait": percentiles([q.t_start - q.t_arrival for q in nq]),
                                                 "build": percentiles([q.t_built - q.t_start for q in nq]),
                                                 "copy_apply_copy": percentiles([q.t_done - q.t_built for q in nq])},
                         "mean_batch": round(float(np.mean([f.request.batch for f in futs])), 2),
                         "server": {k: v for k, v in srv.stats().items() if k != "budget"}}
    torch.cuda.synchronize()
    # plain path: the same requests one call at a time (build, copy in, apply, copy out, free)
    for mode in ("plain_per_call", "plain_cached"):
        store = {}
        t0 = time.perf_counter()
        lat = []
        from regridding_gb300 import _device
        for i, r in enumerate(reqs):
            s = time.perf_counter()
            gi, go = r["pair"]
            if mode == "plain_per_call" or r["cached"] < 0:
                regrid_plain(gi, go, values(r), out=sink(i, r), perturb=False)
            else:
                dw = store.get(r["cached"])
                if dw is None:
                    dw = store[r["cached"]] = _device.build_conservative_2d(gi, go)
                v = values(r).cuda(non_blocking=True)
                o = dw.apply(v, accumulate="fast")
                sink(i, r).copy_(o)
            lat.append(time.perf_counter() - s)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        p50, p99 = percentiles(lat)
        out[mode] = {"req_per_s": round(n_req / t, 1), "service_p50_ms": p50, "service_p99_ms": p99}
        for dw in store.values():
            dw.free()
    out["speedup_saturated_vs_plain_per_call"] = round(out["saturated"]["req_per_s"] /
                                                        out["plain_per_call"]["req_per_s"], 2)
    # what the upstream's default server-side jitter would add per new grid
    # (numpy normal() on the host, one core)
    from regridding_gb300 import _util
    news = [r for r in reqs if r["cached"] < 0][:20]
    s = time.perf_counter()
    for r in news:
        _util.normalize_input_output_coordinates(*r["pair"], None, None, perturb=True, seed=42)
    out["host_jitter_ms_per_new_grid"] = round((time.perf_counter() - s) / len(news) * 1e3, 2)
    out["weights_check"] = served_weights_check(reqs, cells)
    return out


def served_weights_check(reqs, cells):
    """Weights of new grids of the served stream against the oracle (float64
    sweep + coalesce on every host core): the new grid at every size decile
    (0, 10, ..., 90 %) and the largest one, built as the server builds them."""
    import oracle
    from regridding_gb300 import _device

    new = sorted((r for r in reqs if r["cached"] < 0), key=lambda r: cells(r["pair"][0]))
    picks = sorted({int(q * (len(new) - 1) / 10) for q in range(10)} | {len(new) - 1})
    rows = []
    for k in picks:
        gi, go = new[k]["pair"]
        dw = _device.build_conservative_2d(gi, go)
        got = dw.export_numpy()
        dw.free()
        exp = oracle.weights_conservative_2d(gi, go)
        same = all(np.array_equal(a, b) for a, b in zip(got, exp))
        if same:
            rel = 0.0
        elif got[2].shape == exp[2].shape and all(np.array_equal(a, b) for a, b in zip(got[:2], exp[:2])):
            rel = float(np.max(np.abs(got[2] - exp[2]) / np.maximum(np.abs(exp[2]), 1e-300)))
        else:
            rel = float("inf")
        rows.append({"side": int(gi[0].shape[0] - 1), "nnz": int(exp[2].size), "bit_identical": same,
                     "max_rel_err": rel})
    return {"grids": rows,
            "summary": {"grids": len(rows), "bit_identical": sum(r["bit_identical"] for r in rows),
                        "max_rel_err": max(r["max_rel_err"] for r in rows),
                        "sides": [r["side"] for r in rows]}}


def run_conservative_1d(args, torch):
    """Per-spectrum 1D conservative weights at scale (the next item after the
    2D path): 10^5 spectra, each with its own sorted input grid of 1025 edges
    and output grid of 769 edges, through the public weights() (saved layout:
    one element per spectrum); the CPU oracle builds a 10^3-spectrum sample."""
    import oracle
    import regridding_gb300 as rg

    rng = np.random.default_rng(14)
    nd, m, n = (10_000 if getattr(args, "small", False) else 100_000), 1025, 769
    x_in = np.sort(rng.uniform(0, 1, (nd, m)), axis=1)
    x_out = np.sort(rng.uniform(0, 1, (nd, n)), axis=1)
    ts = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        w, _, _ = rg.weights(x_in, x_out, axis_input=1, axis_output=1, method="conservative")
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    same = all(all(np.array_equal(a, b) for a, b in zip(w[k], oracle.conservative_1d(x_in[k], x_out[k])))
               for k in (0, 1, nd // 2, nd - 1))
    t0 = time.perf_counter()
    for k in range(1000):
        oracle.conservative_1d(x_in[k], x_out[k])
    t_cpu = time.perf_counter() - t0
    return {"workload": f"1D conservative, {nd} spectra, 1025 -> 769 edges each, per-spectrum grids",
            "weights_ms": round(min(ts) * 1e3, 1), "spectra_per_s": round(nd / min(ts), 0),
            "bit_identical_to_oracle_sample": same,
            "cpu_baseline": {"spectra_per_s": round(1000 / t_cpu, 0), "cores": 1, "kind": "port",
                             "sample": "10^3 spectra, one thread"}}


def run_batched(args, torch):
    """256 uneven grid pairs (sides log-uniform in [64, 1024] cells, random
    rotation and sinusoidal distortion of amplitude uniform(0, 0.03), output
    rectilinear over 90-110 % of the input extent at 0.75x the side), float32
    Poisson(50) stacks of depth 1, 4 or 16: the batched build against the same
    pairs built one call at a time, and the applies replayed through one CUDA
    graph against the same applies launched one by one."""
    from regridding_gb300 import _device, batching, workloads

    t0 = time.perf_counter()
    pairs, stacks = workloads.batched_pairs(32 if getattr(args, "small", False) else 256)
    t_gen = time.perf_counter() - t0
    cells = sum((gi[0].shape[0] - 1) * (gi[0].shape[1] - 1) + (go[0].shape[0] - 1) * (go[0].shape[1] - 1)
                for gi, go in pairs)
    dev = [(tuple(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in gi),
            tuple(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in go)) for gi, go in pairs]
    torch.cuda.synchronize()
    # one call at a time
    t0 = time.perf_counter()
    single = [_device.build_conservative_2d(gi, go) for gi, go in dev]
    torch.cuda.synchronize()
    t_single = time.perf_counter() - t0
    for w in single:
        w.free()
    # batched (warm-up call first: device memory pool)
    for w in batching.build_batch(dev[:8]):
        w.free()
    torch.cuda.synchronize()
    ts = []
    built = None
    for _ in range(2):
        if built is not None:
            for w in built:
                w.free()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        built = batching.build_batch(dev)
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    t_batch = min(ts)
    failed = sum(1 for w in built if not isinstance(w, _device.DeviceWeights))
    # applies: eager one by one vs one graph replay
    g = torch.Generator(device="cuda")
    g.manual_seed(11)
    items = []
    for dw, st in zip(built, stacks):
        rate = torch.full((st, dw.n_in), 50.0, device="cuda")
        v = torch.poisson(rate, generator=g).to(torch.float32)
        items.append((dw, v, torch.empty((st, dw.n_out), dtype=torch.float32, device="cuda")))
    graph = batching.ApplyGraph(items)
    nbytes = sum(v.numel() * 4 + o.numel() * 4 + dw.nnz * 8 for dw, v, o in items)

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps / 1e3

    t_eager = timed(graph.eager)
    t_graph = timed(graph.replay)
    return {"workload": f"{len(pairs)} uneven grid pairs, sides 64-1024 cells, stacks {{1, 4, 16}} float32 Poisson(50)",
            "input_plus_output_cells": cells, "generation_s": round(t_gen, 2), "failed_pairs": failed,
            "build_batched_ms": round(t_batch * 1e3, 2), "build_one_by_one_ms": round(t_single * 1e3, 2),
            "build_batched_cells_per_s": round(cells / t_batch, 0),
            "build_speedup": round(t_single / t_batch, 2),
            "apply_graph_ms": round(t_graph * 1e3, 3), "apply_eager_ms": round(t_eager * 1e3, 3),
            "apply_graph_GB_per_s": round(nbytes / t_graph / 1e9, 1)}


def run_multilinear_1d(args, torch):
    """The 1D case of the 2048^2 configuration: multilinear weights from a
    shared non-uniform sorted axis of 4096 samples (sorted uniform(0, 1)) to
    4096 sorted output points, applied to 10^6 float32 spectra (16.4 GB in,
    16.4 GB out, resident in HBM); the CPU oracle applies the same weights
    to a 10^4-spectrum sample."""
    import oracle
    import regridding_gb300 as rg
    from regridding_gb300 import _device

    rng = np.random.default_rng(12)
    x_in = np.sort(rng.uniform(0, 1, 4096))
    x_out = np.sort(rng.uniform(x_in[0], x_in[-1], 4096))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    w, shape_in, shape_out = rg.weights(x_in, x_out, method="multilinear")
    t_w = time.perf_counter() - t0
    ii, oo, vv = w[()] if w.shape == () else w.reshape(-1)[0]
    dw = _device.DeviceWeights.from_coo(ii, oo, vv, 4096, 4096)
    n_spec = 50_000 if getattr(args, "small", False) else 1_000_000
    g = torch.Generator(device="cuda")
    g.manual_seed(13)
    vals = torch.rand((n_spec, 4096), generator=g, device="cuda", dtype=torch.float32)
    out = torch.empty((n_spec, 4096), dtype=torch.float32, device="cuda")
    per, wall = time_launches(lambda: dw.apply(vals, out=out, accumulate="fast"), 5, 3, torch.cuda.current_stream(),
                              torch)
    nbytes = apply_bytes(n_spec, 4096, 4096, dw.nnz)
    # parity on a sample of spectra against the oracle's float64 apply
    sample = vals[:2048].cpu().numpy()
    exp = oracle.apply(ii, oo, vv, sample.astype(np.float64), 4096)
    rel = float(np.max(np.abs(out[:2048].cpu().numpy() - exp) / np.maximum(np.abs(exp), 1e-30)))
    # CPU oracle on 10^4 spectra
    host = vals[:10_000].cpu().numpy()
    t0 = time.perf_counter()
    oracle.apply(ii, oo, vv, host, 4096)
    t_cpu = time.perf_counter() - t0
    del vals, out
    return {"workload": f"1D multilinear, 4096 -> 4096 samples, {n_spec} float32 spectra", "nnz": int(dw.nnz),
            "weights_ms": round(t_w * 1e3, 2), "apply_ms": round(statistics.mean(per) * 1e3, 3),
            "apply_GB_per_s": round(nbytes / statistics.mean(per) / 1e9, 1),
            "spectra_per_s": round(n_spec / statistics.mean(per), 0), "max_rel_err_vs_f64_sample": rel,
            "cpu_baseline": {"spectra_per_s": round(10_000 / t_cpu, 0), "cores": os.cpu_count(),
                             "kind": "port", "sample": "10^4 spectra, float64 output"}}


def run_interp(args, torch):
    """ndarray_linear_interpolation of a 16-deep float64 stack of 2048^2
    samples at the 2048^2 points of the sample grid rotated by 0.1 rad and
    scaled by 0.95 about its centre (one set of points for all slices): the
    kernel on resident device buffers (algorithmic bytes: the stack, the two
    index arrays once, the result), and the public call from host arrays.
    The CPU oracle interpolates one slice."""
    import oracle
    import regridding_gb300 as rg
    from regridding_gb300 import _device, _lib

    n, depth = 2048, (4 if getattr(args, "small", False) else 16)
    g = torch.Generator(device="cuda")
    g.manual_seed(15)
    a = torch.rand((depth, n, n), generator=g, device="cuda", dtype=torch.float64)
    i, j = np.meshgrid(np.arange(n, dtype=np.float64), np.arange(n, dtype=np.float64), indexing="ij")
    c, s_, mid = 0.95 * np.cos(0.1), 0.95 * np.sin(0.1), (n - 1) / 2
    x = (mid + c * (i - mid) - s_ * (j - mid))[None]
    y = (mid + s_ * (i - mid) + c * (j - mid))[None]
    dx, dy = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    out = torch.empty((depth, n * n), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()

    def launch():
        _lib.call("rg_interp_linear", _device.ptr(a), n * n, n, n, _device.ptr(dx), _device.ptr(dy), 0, n * n, depth,
                  _device.ptr(out), _device.stream())

    per, _ = time_launches(launch, 20, 3, stream, torch)
    nbytes = (2 * depth + 2) * n * n * 8
    peak, _ = measured_peak()
    host_a = a.cpu().numpy()
    ts = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = rg.ndarray_linear_interpolation(host_a, (x, y), axis=(1, 2), axis_indices=(1, 2))
        ts.append(time.perf_counter() - t0)
    t0 = time.perf_counter()
    exp0 = oracle.ndarray_linear_interpolation(host_a[:1], (x, y), axis=(1, 2), axis_indices=(1, 2))
    t_cpu = time.perf_counter() - t0
    exp_last = oracle.ndarray_linear_interpolation(host_a[-1:], (x, y), axis=(1, 2), axis_indices=(1, 2))
    same = bool(np.array_equal(res[:1], exp0) and np.array_equal(res[-1:], exp_last)
                and np.array_equal(out[0].cpu().numpy(), exp0.reshape(-1)))
    del a, out, dx, dy
    return {"workload": f"bilinear interpolation, {depth} x 2048^2 float64 samples at 2048^2 rotated points",
            "kernel_ms": round(statistics.mean(per) * 1e3, 4),
            "kernel_GB_per_s": round(nbytes / statistics.mean(per) / 1e9, 1),
            "frac_of_measured_hbm": round(nbytes / statistics.mean(per) / 1e9 / peak, 3),
            # bound: the FP64 pipe (2 operations per clock per SM, 152 SMs): 4 products and 3
            # sums per value plus the 8-operation weights of a point shared by all slices
            "fp64_ops_per_value": 7 + 8 / depth,
            "frac_of_fp64_peak_at_2070MHz": round(depth * n * n * (7 + 8 / depth) / statistics.mean(per)
                                                  / (152 * 2 * 2.07e9), 3),
            "public_call_ms": round(min(ts) * 1e3, 2), "bit_identical_to_oracle": same,
            "cpu_baseline": {"points_per_s": round(n * n / t_cpu, 0), "cores": 1, "kind": "port",
                             "sample": "one 2048^2 slice, numpy"}}


def run_fill(args, torch):
    """fill(method="gauss_seidel") of a 64 x 1024^2 float64 stack with 200
    random rectangular holes (4-40 cells a side) per slice (8.4 % of the
    cells missing), median guess, 100 iterations: the whole device path
    (median, seeding, list compaction, 200 relaxation launches) on resident
    buffers, and the public call from host arrays.  The CPU oracle fills one
    slice."""
    import oracle
    import regridding_gb300 as rg
    from regridding_gb300 import _device, _lib

    rng = np.random.default_rng(40)
    nt, ny, nx, iters = 64, 1024, 1024, 100
    if getattr(args, "small", False):
        nt, iters = 16, 3
    a = rng.normal(0, 1, (nt, ny, nx))
    where = np.zeros(a.shape, bool)
    for t in range(nt):
        for _ in range(200):
            j, i = rng.integers(0, ny - 40), rng.integers(0, nx - 40)
            where[t, j:j + rng.integers(4, 40), i:i + rng.integers(4, 40)] = True
    missing = int(where.sum())
    d_a0 = _device.upload(a)
    d_w = _device.upload(where.view(np.uint8))

    def run(n_iter):
        d_a = d_a0.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _lib.call("rg_fill_gauss_seidel", _device.ptr(d_a), _lib.RG_F64, _device.ptr(d_w), nt, ny, nx, None,
                  _lib.RG_FILL_GUESS_MEDIAN, n_iter, _device.stream())
        torch.cuda.synchronize()
        return time.perf_counter() - t0, d_a

    for _ in range(2):
        run(iters)
    t_full = min(run(iters)[0] for _ in range(3))
    t_seed = min(run(0)[0] for _ in range(3))
    _, d_out = run(iters)
    per_iter = (t_full - t_seed) / iters
    t0 = time.perf_counter()
    res = rg.fill(a, where=where, axis=(1, 2), num_iterations=iters)
    t_public = time.perf_counter() - t0
    t0 = time.perf_counter()
    exp0 = oracle.fill(a[:1], where=where[:1], axis=(1, 2), num_iterations=iters)
    t_cpu = time.perf_counter() - t0
    same = bool(np.array_equal(res[:1], exp0) and np.array_equal(d_out[0].cpu().numpy(), exp0[0]))
    del d_a0, d_w, d_out
    return {"workload": f"fill, {nt} x 1024^2 float64, {100 * missing / where.size:.1f} % missing in rectangular "
                        f"holes, median guess, {iters} iterations",
            "missing_cells": missing, "device_ms": round(t_full * 1e3, 2),
            "median_and_seed_ms": round(t_seed * 1e3, 2), "iteration_us": round(per_iter * 1e6, 1),
            "cell_updates_per_s": round(missing * iters / (t_full - t_seed), 0),
            # bound: the FP64 pipe (2 operations per clock per SM, 152 SMs), 6 operations per update
            "frac_of_fp64_peak_at_2070MHz": round(missing * 6 / per_iter / (152 * 2 * 2.07e9), 3),
            "public_call_ms": round(t_public * 1e3, 1), "bit_identical_to_oracle_slice": same,
            "cpu_baseline": {"cell_updates_per_s": round(int(where[0].sum()) * iters / t_cpu, 0), "cores": 1,
                             "kind": "port", "sample": f"one 1024^2 slice, {iters} iterations, sequential C"}}


def run_find_indices_2d(args, torch):
    """2D find_indices (the lowest-index input cell holding each point) of
    the output vertices of the 2048^2 -> 1536^2 grids (sizes from --n-in and
    --n-out) by the grid walk, on resident device arrays; a 20,000-point
    sample is checked against the oracle's secant locate."""
    import oracle
    import regridding_gb300 as rg
    from regridding_gb300 import workloads

    gi, go = workloads.cfg2_grids(args.n_in, args.n_out)
    gop = workloads.perturb(go)
    d_gi = tuple(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in gi)
    px = torch.from_numpy(np.ascontiguousarray(gop[0]).reshape(-1)).cuda()
    py = torch.from_numpy(np.ascontiguousarray(gop[1]).reshape(-1)).cuda()
    ts = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        oi, oj = rg.locate_2d(d_gi, px, py, method="brute")
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    pick = np.random.default_rng(1).choice(px.numel(), 20_000, replace=False)
    exp = oracle.locate(gi, gop[0].reshape(-1)[pick], gop[1].reshape(-1)[pick], "secant")
    same = bool(np.array_equal(oi.cpu().numpy()[pick], exp[0]) and np.array_equal(oj.cpu().numpy()[pick], exp[1]))
    return {"workload": f"{px.numel()} output vertices in the {args.n_in - 1}^2-cell quadratic-mapped grid",
            "ms": [round(t * 1e3, 3) for t in ts], "points_per_s": round(px.numel() / min(ts), 0),
            "outside": int((oi == np.iinfo(np.int64).max).sum().item()), "sample_equals_oracle": same}


def run_differentiable(args, torch):
    """One optimisation step of the differentiable regrid: 1024^2 -> 768^2
    cells, 16 float32 N(0, 1) slices, output coordinates learnable (a
    rectilinear grid on [-0.95, 0.95]^2 plus N(0, 1e-4) jitter), loss = squared
    error against the values regridded onto the output grid rotated by
    0.05 rad.  A step is forward (weights build + apply) and backward (values
    gradient by the transposed apply, coordinate gradient by the overlap-area
    adjoint)."""
    from regridding_gb300 import workloads
    from regridding_gb300.autograd import regrid_conservative_2d

    gi, go, gt = workloads.cfg4_grids()
    g = torch.Generator(device="cuda")
    g.manual_seed(4)
    v = torch.randn((16, 1024, 1024), generator=g, device="cuda").requires_grad_(True)
    d_gi = tuple(torch.from_numpy(a).cuda() for a in gi)
    with torch.no_grad():
        target = regrid_conservative_2d(v, d_gi, tuple(torch.from_numpy(a).cuda() for a in gt))
    xo = torch.from_numpy(go[0].copy()).cuda().requires_grad_(True)
    yo = torch.from_numpy(go[1].copy()).cuda().requires_grad_(True)

    def step():
        v.grad = xo.grad = yo.grad = None
        out = regrid_conservative_2d(v, d_gi, (xo, yo))
        loss = 0.5 * ((out - target) ** 2).sum()
        loss.backward()
        return loss

    for _ in range(2):
        step()
    torch.cuda.synchronize()
    ts = []
    for _ in range(5):
        t0 = time.perf_counter()
        loss = step()
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    return {"workload": "1024^2 -> 768^2 cells, 16 float32 slices, learnable output coordinates",
            "ms_per_step": round(statistics.median(ts) * 1e3, 2), "steps": 5,
            "loss": float(loss.item()), "grad_norm_xy": float(torch.sqrt((xo.grad ** 2).sum() +
                                                                          (yo.grad ** 2).sum()).item()),
            "checks": "tests/test_gpu_autograd.py: FD (float64, h=1e-7) and transposed-weights parity"}


WORKLOAD = ("2048^2 -> 1536^2 conservative apply of a 64-slice float32 log-normal(3, 1) stack, float64 output "
            "as the upstream returns (quadratic-mapped input grid, rectilinear output on [-1.05, 1.05]^2)")
HEADLINE = "apply HBM GB/s: 2048^2 -> 1536^2 conservative weights, 64-deep float32 stack, float64 output"


def bench_config(nnz: int) -> dict:
    """The workload of the headline, identical in both arms."""
    n_in_cells, n_out_cells = (N_IN - 1) ** 2, (N_OUT - 1) ** 2
    return {"workload": WORKLOAD, "stack": STACK, "input_cells": n_in_cells, "output_cells": n_out_cells,
            "nnz": nnz, "output_dtype": "float64",
            "bytes_per_step": apply_bytes(STACK, n_in_cells, n_out_cells, nnz, b_out=8, b_val=8),
            "l2": "inputs (1.07 GB) exceed L2 (129 MB); no flush"}


def run_ours(args, world, rank, local):
    import torch

    import oracle
    import regridding_gb300 as rg
    from regridding_gb300 import _lib, workloads

    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    s_ptr = ctypes.c_void_p(stream.cuda_stream)

    gi, go = workloads.cfg2_grids(N_IN, N_OUT)
    gop = workloads.perturb(go)
    n_in_cells = (N_IN - 1) ** 2
    n_out_cells = (N_OUT - 1) ** 2
    d_gi = tuple(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in gi)
    d_go = tuple(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in gop)

    # --- weight build (each call synchronises to size its buffers)
    build_ms = []
    dw = None
    for _ in range(3):
        if dw is not None:
            dw.free()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dw = rg.build_conservative_2d(d_gi, d_go)
        torch.cuda.synchronize()
        build_ms.append((time.perf_counter() - t0) * 1e3)
    nnz = dw.nnz

    # --- 2D find_indices of the output vertices in the input grid
    px, py = d_go[0].reshape(-1), d_go[1].reshape(-1)
    fi_ms = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        oi, oj = rg.locate_2d(d_gi, px, py, method="brute")
        torch.cuda.synchronize()
        fi_ms.append((time.perf_counter() - t0) * 1e3)
    n_outside = int((oi == np.iinfo(np.int64).max).sum().item())

    # --- applies: compensated float64 output (headline), fast float32, exact float64
    values = workloads.cfg2_values_torch(STACK, N_IN - 1, seed=rank)
    out32 = torch.empty((STACK, n_out_cells), dtype=torch.float32, device="cuda")
    out64 = torch.empty((STACK, n_out_cells), dtype=torch.float64, device="cuda")
    ref64 = torch.empty((STACK, n_out_cells), dtype=torch.float64, device="cuda")
    lib = _lib.load()
    h = dw.handle

    def launcher(out, dtype_out, acc):
        vp, op = ctypes.c_void_p(values.data_ptr()), ctypes.c_void_p(out.data_ptr())

        def fn():
            st = lib.rg_apply(h, vp, _lib.RG_F32, op, dtype_out, STACK, acc, s_ptr)
            if st:
                _lib.check(st, "rg_apply")
        return fn

    apply_comp = launcher(out64, _lib.RG_F64, _lib.RG_ACC_COMPENSATED)
    apply_fast = launcher(out32, _lib.RG_F32, _lib.RG_ACC_FAST)
    apply_exact = launcher(ref64, _lib.RG_F64, _lib.RG_ACC_EXACT)

    cfg = bench_config(nnz)
    bytes_step = cfg["bytes_per_step"]
    bytes_f32 = apply_bytes(STACK, n_in_cells, n_out_cells, nnz)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        per, wall = time_launches(apply_comp, args.steps, args.warmup, stream, torch)
    barrier(world)
    wall_max = aggregate_seconds(wall, world, device="cuda")
    value = world * bytes_step * args.steps / wall_max / 1e9
    kernel_s = statistics.mean(per)

    per32, _ = time_launches(apply_fast, max(5, args.steps), 3, stream, torch)
    per64, _ = time_launches(apply_exact, max(5, args.steps // 4), 2, stream, torch)

    # --- end to end through the C ABI from page-locked host buffers
    h_in = torch.empty((STACK, n_in_cells), dtype=torch.float32, pin_memory=True)
    h_in.copy_(values)
    h_out = torch.empty((STACK, n_out_cells), dtype=torch.float64, pin_memory=True)
    torch.cuda.synchronize()

    def apply_host():
        st = lib.rg_apply_host(h, ctypes.c_void_p(h_in.data_ptr()), _lib.RG_F32, ctypes.c_void_p(h_out.data_ptr()),
                               _lib.RG_F64, STACK, _lib.RG_ACC_COMPENSATED, 0, s_ptr)
        if st:
            _lib.check(st, "rg_apply_host")

    e2e_steps = max(3, min(args.steps, 20))
    per_e2e, wall_e2e = time_launches(apply_host, e2e_steps, 3, stream, torch)
    e2e_value = world * bytes_step * e2e_steps / aggregate_seconds(wall_e2e, world, device="cuda") / 1e9

    # parity at full size: compensated and fast against the exact float64
    # result (bit-identical to the upstream apply), relative per output cell
    apply_comp()
    apply_fast()
    apply_exact()
    torch.cuda.synchronize()
    covered = ref64 != 0
    denom = ref64.abs().clamp_min(1e-300)
    rel64 = float(((out64 - ref64).abs() / denom)[covered].max().item())
    rel32 = float(((out32.double() - ref64).abs() / denom)[covered].max().item())
    host_same = bool(torch.equal(h_out.cuda(), out64))
    # conservation: the output total against the input weighted by the
    # fraction of each input cell the output grid covers (the transposed
    # apply of ones), per slice, relative to the input total
    ones = torch.ones((1, n_out_cells), dtype=torch.float64, device="cuda")
    frac_in = dw.apply(ones, transpose=True, accumulate="exact")[0]
    vin64 = values.double()
    cons = ((out64.sum(1) - vin64 @ frac_in).abs() / vin64.sum(1)).max().item()
    cons_uncovered = float(1.0 - (vin64 @ frac_in).sum().item() / vin64.sum().item())
    del vin64, ones, frac_in, ref64

    # --- CPU baseline: the oracle (C restatement of the upstream loops, all cores)
    cpu = None
    if rank == 0 and not args.no_cpu:
        ii, oo, vv = dw.export_numpy()
        host_vals = h_in.numpy()
        ts = []
        for _ in range(2):
            t0 = time.perf_counter()
            oracle.apply(ii, oo, vv, host_vals, n_out_cells)
            ts.append(time.perf_counter() - t0)
        t_cpu = min(ts)
        cpu = {"value": round(bytes_step / t_cpu / 1e9, 3), "unit": "GB/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"the full 64-slice apply, float64 output as upstream, best of 2 ({t_cpu * 1e3:.1f} ms): "
                         "C restatement of the upstream loop, OpenMP over the stack"}

    peak, peak_kind = measured_peak()
    achieved = bytes_step / kernel_s / 1e9
    achieved32 = bytes_f32 / statistics.mean(per32) / 1e9
    traffic = profiled_traffic("apply_kernel_compensated")
    line = {
        "metric": METRIC,
        "headline": HEADLINE,
        "value": round(value, 2),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(wall_max / args.steps * 1e3, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "float-float (float32 stack, float64 output)",
        "accumulate": "compensated: products split exactly by FMA, sums as float pairs (two-sum), float64 at the "
                      f"end; max relative error against the upstream float64 result {rel64:.2e}",
        "data": "synthetic (seeded grids and log-normal stack generated on the device)",
        "config": cfg,
        "parallelism": f"replicas x{world}",
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": peak_kind,
                     "achieved_basis": "bytes_per_step / mean CUDA-event duration of one launch",
                     "traffic_basis": "dram read + write bytes of one launch from the ncu capture recorded in "
                                      "profiles/traffic.json (not measured in this run)"},
        "cpu_baseline": cpu,
        "e2e": {"value": round(e2e_value, 2), "unit": "GB/s",
                "h2d_bytes_per_step": STACK * n_in_cells * 4, "d2h_bytes_per_step": STACK * n_out_cells * 8,
                "ms_per_step": round(wall_e2e / e2e_steps * 1e3, 3),
                "path": "rg_apply_host (RG_ACC_COMPENSATED), pinned host buffers", "equals_device_result": host_same},
        "gpu_launches": args.steps,
        "clocks": clocks.summary(),
        "apply_f32_fast": {"GB_per_s": round(achieved32, 1), "ms": round(statistics.mean(per32) * 1e3, 4),
                           "frac_of_measured_hbm": round(achieved32 / peak, 4), "bytes_per_step": bytes_f32,
                           "max_rel_err_vs_f64": rel32, "note": "float32 output, float32 FMA accumulation"},
        "apply_f64_exact": {"GB_per_s": round(bytes_step / statistics.mean(per64) / 1e9, 1),
                            "ms": round(statistics.mean(per64) * 1e3, 4),
                            "note": "bit-identical to the upstream float64 apply (FP64-pipe bound)"},
        "conservation": {"max_rel_err": cons, "input_fraction_outside_output_grid": cons_uncovered},
        "build": {"cells_per_s": round((n_in_cells + n_out_cells) / (min(build_ms) / 1e3), 0),
                  "ms": [round(v, 2) for v in build_ms], "nnz": nnz},
        "find_indices_2d": {"points_per_s": round(px.numel() / (min(fi_ms) / 1e3), 0),
                            "ms": [round(v, 3) for v in fi_ms], "points": int(px.numel()),
                            "outside": n_outside},
    }
    del values, out32, out64
    torch.cuda.empty_cache()
    if rank == 0 and args.serve_requests > 0:
        line["serving"] = run_serving(args, torch)
    if rank == 0 and not args.no_extra:
        line["multilinear_1d"] = run_multilinear_1d(args, torch)
        line["conservative_1d"] = run_conservative_1d(args, torch)
        line["batched"] = run_batched(args, torch)
        line["differentiable"] = run_differentiable(args, torch)
        line["interp_2d"] = run_interp(args, torch)
        line["fill"] = run_fill(args, torch)
    if rank == 0:
        line["summary"] = summary_of(line)
        print(json.dumps(line), flush=True)


def summary_of(line: dict) -> dict:
    """The figures of every leg in a few hundred bytes, placed last in the
    line so that a truncated tail of the output still holds them."""
    s = {"apply_f64out_ms": line["ms_per_step"], "apply_f64out_frac": line["roofline"]["frac"],
         "apply_f32_ms": line["apply_f32_fast"]["ms"], "apply_f32_frac": line["apply_f32_fast"]["frac_of_measured_hbm"],
         "apply_exact_ms": line["apply_f64_exact"]["ms"], "build_ms": min(line["build"]["ms"]),
         "e2e_GB_per_s": line["e2e"]["value"]}
    srv = line.get("serving")
    if srv:
        s["serve_poisson_p50_p99_ms"] = [srv["poisson"]["p50_ms"], srv["poisson"]["p99_ms"]]
        s["serve_saturated_req_s"] = srv["saturated"]["req_per_s"]
        s["serve_plain_req_s"] = srv["plain_per_call"]["req_per_s"]
        s["serve_speedup"] = srv["speedup_saturated_vs_plain_per_call"]
        s["serve_weights_check"] = srv.get("weights_check", {}).get("summary")
    if "batched" in line:
        b = line["batched"]
        s["batched_build_ms"] = [b["build_batched_ms"], b["build_one_by_one_ms"]]
        s["batched_apply_graph_GB_per_s"] = b["apply_graph_GB_per_s"]
    if "differentiable" in line:
        s["differentiable_step_ms"] = line["differentiable"]["ms_per_step"]
    if "multilinear_1d" in line:
        s["multilinear_1d_GB_per_s"] = line["multilinear_1d"]["apply_GB_per_s"]
    return s


# ---------------------------------------------------------------------------
# reference arm: the upstream algorithm on the host cores (C restatement)
# ---------------------------------------------------------------------------


def run_reference(args, world, rank):
    if rank != 0:
        return
    import oracle
    from regridding_gb300 import workloads

    gi, go = workloads.cfg2_grids(N_IN, N_OUT)
    gop = workloads.perturb(go)
    n_out_cells = (N_OUT - 1) ** 2
    n_in_cells = (N_IN - 1) ** 2
    t0 = time.perf_counter()
    raw = oracle.sweep_2d(gi, gop)
    t1 = time.perf_counter()
    ii, oo, vv = oracle.coalesce(*raw)
    t2 = time.perf_counter()
    del raw
    nnz = vv.size
    cfg = bench_config(nnz)
    rng = np.random.default_rng(0)
    values = rng.lognormal(3, 1, (STACK, n_in_cells)).astype(np.float32)
    bytes_step = cfg["bytes_per_step"]
    for _ in range(args.warmup):
        oracle.apply(ii, oo, vv, values, n_out_cells)
    ts = []
    for _ in range(args.steps):
        s = time.perf_counter()
        oracle.apply(ii, oo, vv, values, n_out_cells)
        ts.append(time.perf_counter() - s)
    total = sum(ts)
    value = bytes_step * args.steps / total / 1e9
    cores = os.cpu_count()
    line = {
        "metric": METRIC,
        "impl": "reference",
        "headline": HEADLINE,
        "value": round(value, 3),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(total / args.steps * 1e3, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded grids, numpy log-normal stack)",
        "config": cfg,
        "parallelism": f"{cores} host threads",
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": "the full 64-slice apply per step (C restatement of the upstream loop, "
                                   "OpenMP over the stack, float64 accumulation and output as upstream)"},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "build": {"cells_per_s": round((n_in_cells + n_out_cells) / (t2 - t0), 0),
                  "sweep_s": round(t1 - t0, 2), "coalesce_s": round(t2 - t1, 2), "nnz": nnz},
    }
    print(json.dumps(line), flush=True)


LEGS = {
    "multilinear_1d": lambda args, torch: run_multilinear_1d(args, torch),
    "conservative_1d": lambda args, torch: run_conservative_1d(args, torch),
    "batched": lambda args, torch: run_batched(args, torch),
    "differentiable": lambda args, torch: run_differentiable(args, torch),
    "interp_2d": lambda args, torch: run_interp(args, torch),
    "fill": lambda args, torch: run_fill(args, torch),
    "find_indices_2d": lambda args, torch: run_find_indices_2d(args, torch),
    "serving": lambda args, torch: run_serving(args, torch),
}


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", choices=("ours", "reference"), default="ours")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--quick", action="store_true",
                   help="build + fast apply only at --n-in/--n-out/--stack (for profiling)")
    p.add_argument("--n-in", type=int, default=N_IN)
    p.add_argument("--n-out", type=int, default=N_OUT)
    p.add_argument("--stack", type=int, default=STACK)
    p.add_argument("--quick-modes", default="fast,compensated,exact",
                   help="with --quick: accumulation modes to time, in order")
    p.add_argument("--serve-requests", type=int, default=1000, help="requests of the served stream (0: skip)")
    p.add_argument("--serve-slots", type=int, default=16)
    p.add_argument("--serve-cobuild", type=int, default=0, help="small grids built together per build job")
    p.add_argument("--serve-urgent", type=int, default=0, help="1: build jobs on high-priority streams")
    p.add_argument("--serve-switch-ms", type=float, default=0.0, help="GIL switch interval (0: unchanged)")
    p.add_argument("--no-extra", action="store_true", help="skip the differentiable-regrid and batched legs")
    p.add_argument("--only", choices=sorted(LEGS), help="run one secondary leg alone and print its JSON (profiling)")
    p.add_argument("--small", action="store_true",
                   help="with --only: the leg's reduced profiling size (interp_2d, fill, multilinear_1d, "
                        "conservative_1d, batched)")
    args = p.parse_args(argv)
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_env()
    if args.impl == "reference":
        # the CPU reference runs on rank 0 only; other ranks exit at once
        run_reference(args, world, rank)
        return
    if args.quick:
        run_quick(args, local)
        return
    if args.only:
        import torch

        torch.cuda.set_device(local)
        print(json.dumps({args.only: LEGS[args.only](args, torch)}), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group(backend="nccl")
    try:
        run_ours(args, world, rank, local)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    main()
