"""Batched conservative regridding: many uneven grids at once.

* ``build_batch(pairs)`` builds the weights of every (grid_input,
  grid_output) pair together (``rg_build_conservative_2d_batch``): each stage
  of the build is one launch over the lines, chunks and output rows of all
  pairs, with a fixed number of host synchronisations per batch.
* ``ApplyGraph`` replays a fixed set of applies (one per pair, each with its
  own stack) through one captured CUDA graph: after a first eager pass (which
  makes every handle's lazily built state and runs the apply autotuner) the
  whole set is a single graph launch.
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
    results written to, the same tensors at every replay."""

    def __init__(self, items, accumulate: str = "fast"):
        torch = _device.torch()
        self.items = list(items)
        self.accumulate = accumulate
        # eager pass: lazily built per-handle state and the apply autotuner
        for dw, v, o in self.items:
            dw.apply(v, out=o, accumulate=accumulate)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            with torch.cuda.graph(self.graph, stream=side):
                for dw, v, o in self.items:
                    dw.apply(v, out=o, accumulate=accumulate)
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
