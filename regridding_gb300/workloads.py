"""Seeded synthetic grids and value stacks for the benchmark configurations.

The upstream publishes no datasets for its benchmarks; these generators make
grids with the stated shapes and distortions from fixed numpy seeds, so every
run (and the CPU baseline) sees identical inputs.
"""

from __future__ import annotations

import numpy as np

SEED_GEOMETRY = 2
"""Seed of the cfg2 rotation angle and quadratic-map coefficients."""


def distorted_grid(n: int, angle: float, amp: float, lo: float = -1.0, hi: float = 1.0):
    """``n x n`` vertices on ``[lo, hi]^2`` rotated by ``angle``, then
    ``x += amp sin(pi y)`` followed by ``y += amp sin(pi x)`` (the second
    uses the updated x).  This is the 65^2 (0.1 rad, 0.02) small-grid
    workload and the sinusoidal family of the batched configuration."""
    a = np.linspace(lo, hi, n)
    x, y = np.meshgrid(a, a, indexing="ij")
    xr = x * np.cos(angle) - y * np.sin(angle)
    yr = x * np.sin(angle) + y * np.cos(angle)
    xr = xr + amp * np.sin(np.pi * yr)
    yr = yr + amp * np.sin(np.pi * xr)
    return xr, yr


def rect_grid(n: int, lo: float, hi: float, m: int | None = None):
    """Rectilinear ``n x m`` vertex grid on ``[lo, hi]^2`` (``indexing="ij"``)."""
    a = np.linspace(lo, hi, n)
    b = np.linspace(lo, hi, n if m is None else m)
    return tuple(np.meshgrid(a, b, indexing="ij"))


def quadratic_grid(n: int, seed: int = SEED_GEOMETRY):
    """``n x n`` vertices on ``[-1, 1]^2`` rotated by ``uniform(0, 0.5)`` rad
    and distorted by a quadratic polynomial map ``x' = x + sum_k c_k m_k(x, y)``
    over the monomials (1, x, y, x^2, xy, y^2) with ``c_k ~ N(0, 0.01)``
    drawn independently for each coordinate (the 2048^2 workload)."""
    rng = np.random.default_rng(seed)
    a = np.linspace(-1, 1, n)
    x, y = np.meshgrid(a, a, indexing="ij")
    angle = rng.uniform(0, 0.5)
    xr = x * np.cos(angle) - y * np.sin(angle)
    yr = x * np.sin(angle) + y * np.cos(angle)
    cx = rng.normal(0, 0.01, 6)
    cy = rng.normal(0, 0.01, 6)
    mono = np.stack([np.ones_like(xr), xr, yr, xr * xr, xr * yr, yr * yr])
    return xr + np.tensordot(cx, mono, 1), yr + np.tensordot(cy, mono, 1)


def perturb(grid, seed: int = 42):
    """The default output-grid perturbation of ``weights(method="conservative")``:
    ``default_rng(seed).normal(c, ptp(c) * 1e-9)`` per coordinate, x then y."""
    rng = np.random.default_rng(seed)
    return tuple(rng.normal(c, np.ptp(c) * 1e-9) for c in grid)


def cfg1():
    """65^2 -> 49^2 conservative regrid of 8 Poisson(100) float64 arrays."""
    gi = distorted_grid(65, 0.1, 0.02)
    go = rect_grid(49, -1.1, 1.1)
    values = np.random.default_rng(42).poisson(100, (8, 64, 64)).astype(np.float64)
    return gi, go, values


def cfg2_grids(n_in: int = 2049, n_out: int = 1537):
    """2048^2 -> 1536^2 grids: quadratic-mapped input, rectilinear output on
    [-1.05, 1.05]^2."""
    return quadratic_grid(n_in), rect_grid(n_out, -1.05, 1.05)


def cfg2_values_torch(stack: int = 64, n: int = 2048, seed: int = 0, device="cuda"):
    """float32 log-normal(3, 1) stack generated on the device (seeded)."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    v = torch.empty((stack, n * n), dtype=torch.float32, device=device)
    v.normal_(mean=3.0, std=1.0, generator=g)
    return v.exp_()


def cfg4_grids(n_in: int = 1025, n_out: int = 769, seed: int = 9):
    """The differentiable-regrid workload: input ``n_in x n_in`` vertices on
    [-1, 1]^2 with sinusoidal distortion of amplitude 0.02 (no rotation);
    output a rectilinear ``n_out x n_out`` grid on [-0.95, 0.95]^2 plus
    N(0, 1e-4) vertex jitter (the initial value of the learnable output
    coordinates); the target grid is the output grid rotated by 0.05 rad.
    Returns (grid_input, grid_output, grid_target)."""
    rng = np.random.default_rng(seed)
    gi = distorted_grid(n_in, 0.0, 0.02)
    go = tuple(c + rng.normal(0, 1e-4, c.shape) for c in rect_grid(n_out, -0.95, 0.95))
    c, s = np.cos(0.05), np.sin(0.05)
    gt = (c * go[0] - s * go[1], s * go[0] + c * go[1])
    return gi, go, gt


def grid_pair(rng: np.random.Generator, side: int, jitter: bool = True):
    """One grid pair of the batched and served configurations: an input of
    ``side x side`` cells on [-1, 1]^2 with a random rotation in [0, 0.5) rad
    and sinusoidal distortion of amplitude uniform(0, 0.03); a rectilinear
    output covering uniform(0.9, 1.1) of the input extent with
    ``round(0.75 side)`` cells per axis.  With ``jitter`` the output vertices
    carry a normal(0, ptp * 1e-9) jitter drawn from ``rng`` (the client-side
    form of the upstream's default perturbation: without it the two grids
    share the vertex (0, 0) whenever both vertex counts are odd, and the
    upstream sweep does not terminate on shared vertices).  Vertex arrays are
    read-only."""
    angle = rng.uniform(0, 0.5)
    amp = rng.uniform(0, 0.03)
    gi = distorted_grid(side + 1, angle, amp)
    ext = rng.uniform(0.9, 1.1)
    m = max(1, int(round(0.75 * side)))
    go = rect_grid(m + 1, -ext, ext)
    if jitter:
        go = tuple(rng.normal(c, np.ptp(c) * 1e-9) for c in go)
    for a in (*gi, *go):
        a.setflags(write=False)
    return gi, go


def log_uniform_side(rng: np.random.Generator, lo: int, hi: int) -> int:
    return int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))


def served_stream(n_requests: int, rate: float = 500.0, n_cached: int = 32, reuse: float = 0.7,
                  side_lo: int = 128, side_hi: int = 2048, stacks=(1, 8, 64), seed: int = 5):
    """The served request stream: Poisson arrivals at ``rate`` req/s, grid
    sides log-uniform in [side_lo, side_hi] cells, a fraction ``reuse`` of the
    requests on one of ``n_cached`` grid pairs (weights resident once built),
    the rest on a new grid pair each, stack depths uniform over ``stacks``.

    Returns (cached pairs, requests); a request is a dict with ``t`` (arrival
    offset, s), ``pair`` (the grid pair), ``cached`` (index or -1) and
    ``stack``."""
    rng = np.random.default_rng(seed)
    cached = [grid_pair(rng, log_uniform_side(rng, side_lo, side_hi)) for _ in range(n_cached)]
    t = 0.0
    reqs = []
    for _ in range(n_requests):
        t += rng.exponential(1.0 / rate)
        stack = int(rng.choice(stacks))
        if rng.random() < reuse:
            k = int(rng.integers(n_cached))
            reqs.append({"t": t, "pair": cached[k], "cached": k, "stack": stack})
        else:
            reqs.append({"t": t, "pair": grid_pair(rng, log_uniform_side(rng, side_lo, side_hi)), "cached": -1,
                         "stack": stack})
    return cached, reqs


def batched_pairs(n: int = 256, side_lo: int = 64, side_hi: int = 1024, seed: int = 3):
    """The batched configuration: ``n`` grid pairs (``grid_pair``) with sides
    log-uniform in [side_lo, side_hi] cells, and per pair a stack depth drawn
    from {1, 4, 16}.  Returns (pairs, stacks)."""
    rng = np.random.default_rng(seed)
    pairs, stacks = [], []
    for _ in range(n):
        pairs.append(grid_pair(rng, log_uniform_side(rng, side_lo, side_hi)))
        stacks.append(int(rng.choice((1, 4, 16))))
    return pairs, stacks
