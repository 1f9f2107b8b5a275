"""Batched conservative regridding: many uneven grids at once.

* ``build_batch(pairs)`` builds the weights of every (grid_input,
  grid_output) pair together (``rg_build_conservative_2d_batch``): each stage
  of the build is one launch over the lines, chunks and output rows of all
  pairs, with a fixed number of host synchronisations per batch.
* ``ApplyGraph`` replays a fixed set of applies (one per pair, each with its
  own stack) through one captured CUDA graph: after a first eager pass (which
  makes every handle's lazily built state and runs the apply autotuner) the
  whole set is a single graph launch, its applies in parallel chains.
* ``autotune_sweep_chunk`` times the build of a sample batch for several
  chunk lengths of the parallel walk and keeps the fastest
  (``rg_set_sweep_chunk``); the apply kernels tune themselves per handle.

The upstream builds and applies one element at a time in Python loops
(regridding/_weights/_weights_conservative.py:110-139,
regridding/_regrid/_regrid_from_weights.py:150-162).
"""

from __future__ import annotations

import time

from . import _device, _lib

__all__ = ["build_batch", "ApplyGraph", "autotune_sweep_chunk"]


def build_batch(pairs, weights_input=None, max_cells: int = 48_000_000):
    """DeviceWeights (or the RegridError of a failed pair) for every pair."""
    return _device.build_conservative_2d_batch(pairs, weights_input, max_cells)


class ApplyGraph:
    """A fixed list of applies ``(weights, values, out)`` (device tensors of
    shape ``(stack, n_in)`` and ``(stack, n_out)``) captured once into a CUDA
    graph and replayed with :meth:`replay`.  Inputs are read from, and
    results written to, the same tensors at every replay.

    The applies are independent, so the graph holds them as ``branches``
    parallel chains (the capturing stream forks to side streams through
    events and joins them at the end); each apply goes to the chain with the
    fewest bytes so far, largest first.  Small applies then run side by side
    instead of one after another.  Every apply computes what it computes
    alone, so the results do not depend on ``branches``."""

    def __init__(self, items, accumulate: str = "fast", branches: int = 8):
        torch = _device.torch()
        self.items = list(items)
        self.accumulate = accumulate
        # eager pass: lazily built per-handle state and the apply autotuner
        for dw, v, o in self.items:
            dw.apply(v, out=o, accumulate=accumulate)
        torch.cuda.synchronize()
        self.branches = max(1, min(int(branches), len(self.items)))
        nbytes = [v.numel() * v.element_size() + o.numel() * o.element_size() + dw.nnz * 12
                  for dw, v, o in self.items]
        chains = [[] for _ in range(self.branches)]
        load = [0] * self.branches
        for k in sorted(range(len(self.items)), key=lambda k: -nbytes[k]):
            c = load.index(min(load))
            chains[c].append(k)
            load[c] += nbytes[k]
        self.chains = [sorted(c) for c in chains]
        self.graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        forks = [torch.cuda.Stream() for _ in range(self.branches - 1)]
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            with torch.cuda.graph(self.graph, stream=side):
                fork = torch.cuda.Event()
                fork.record(side)
                streams = [side] + forks
                for st in forks:
                    st.wait_event(fork)
                for st, chain in zip(streams, self.chains):
                    with torch.cuda.stream(st):
                        for k in chain:
                            dw, v, o = self.items[k]
                            dw.apply(v, out=o, accumulate=accumulate)
                for st in forks:
                    join = torch.cuda.Event()
                    join.record(st)
                    side.wait_event(join)
        torch.cuda.current_stream().wait_stream(side)

    def replay(self) -> None:
        self.graph.replay()

    def eager(self) -> None:
        """The same applies launched one by one (the path the graph replaces)."""
        for dw, v, o in self.items:
            dw.apply(v, out=o, accumulate=self.accumulate)


def autotune_sweep_chunk(pairs, candidates=(8, 16, 32, 64, 128), repeats: int = 1) -> dict:
    """Time the batched build of ``pairs`` for every chunk length, keep the
    fastest for the process and return ``{length: seconds}``."""
    torch = _device.torch()
    timings = {}
    for ch in candidates:
        _lib.call("rg_set_sweep_chunk", int(ch))
        best = None
        for _ in range(repeats):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            built = build_batch(pairs)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            for w in built:
                if isinstance(w, _device.DeviceWeights):
                    w.free()
            best = dt if best is None else min(best, dt)
        timings[int(ch)] = best
    choice = min(timings, key=timings.get)
    _lib.call("rg_set_sweep_chunk", choice)
    return timings
