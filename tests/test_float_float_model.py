"""The float-float step of the compensated apply, restated in float32
arithmetic on the host (no GPU): the arithmetic facts the kernel relies on.

Each half of the packed step (``ff_step2`` in
``regridding_gb300/csrc/apply_tiled.cu``) is Dekker's product, split exactly
by an FMA, and Knuth's two-sum, written with ``pn = x * (-wh)`` so that no
operand needs negating.  Checked here:

* the pair ``(h, l)``, widened and added once in float64, is within
  ``(1.5 * 2^-47 + (n + 2)^2 * 2^-48) * sum_k |w_k x_k|`` of the exact sum of
  a row of n entries (the weights split as ``hi = (float)w``,
  ``lo = (float)(w - hi)``);
* a step with zero weights, which lanes take past the end of their own row
  (every lane of a warp runs to the warp's longest row), leaves ``(h, l)``
  unchanged bit for bit for every finite input word, and makes the sum NaN
  for an infinite or NaN word: the kernel then recomputes that output in
  float64 in stored order, as it does for any non-finite input.
"""

from fractions import Fraction

import numpy as np

F = np.float32


def round_f32(q: Fraction) -> np.float32:
    """The float32 nearest to q (ties to even), for |q| below the float32
    maximum."""
    if q == 0:
        return F(0.0)
    sign = -1.0 if q < 0 else 1.0
    q = abs(q)
    e = q.numerator.bit_length() - q.denominator.bit_length()
    if Fraction(2) ** e > q:
        e -= 1
    quantum = max(e - 23, -149)  # 24 significant bits; subnormal spacing 2^-149
    scaled = q / Fraction(2) ** quantum
    n = scaled.numerator // scaled.denominator
    rest = scaled - n
    if rest > Fraction(1, 2) or (rest == Fraction(1, 2) and n % 2 == 1):
        n += 1
    return F(sign * n * 2.0**quantum)


def fma(a, b, c) -> np.float32:
    """float32 fma: a * b + c rounded once."""
    if not (np.isfinite(a) and np.isfinite(b) and np.isfinite(c)):
        return F(np.float64(a) * np.float64(b) + np.float64(c))
    return round_f32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def ff_step(h, l, x, wh, wl):
    """One half of ff_step2: (h, l) += x * (wh + wl)."""
    with np.errstate(invalid="ignore", over="ignore"):
        pn = F(x * F(-wh))
        e = fma(x, wh, pn)
        r = fma(x, wl, e)
        t = F(h - pn)
        bp = F(t - h)
        err = F(F(h - F(t - bp)) - F(pn + bp))
        return t, F(l + F(err + r))


def split(w: float):
    hi = F(w)
    return hi, F(w - float(hi))


def bits(v) -> int:
    return int(np.asarray(v, np.float32).view(np.uint32))


def row_sum(ws, xs):
    h, l = F(0.0), F(0.0)
    for w, x in zip(ws, xs):
        h, l = ff_step(h, l, x, *split(w))
    return h, l


def test_forward_error_bound():
    rng = np.random.default_rng(7)
    worst = 0.0
    for trial in range(400):
        n = int(rng.integers(1, 15))
        ws = rng.uniform(0.0, 1.0, n) ** 3
        xs = rng.lognormal(3, 1, n).astype(np.float32)
        if trial % 4 == 3:  # cancellation: mixed signs of inputs and weights
            xs *= rng.choice([-1, 1], n).astype(np.float32)
            ws *= rng.choice([-1, 1], n)
        h, l = row_sum(ws, xs)
        got = Fraction(float(h) + float(l))
        exact = sum(Fraction(float(w)) * Fraction(float(x)) for w, x in zip(ws, xs))
        scale = sum(abs(Fraction(float(w)) * Fraction(float(x))) for w, x in zip(ws, xs))
        bound = (Fraction(3, 2) * Fraction(1, 2**47) + (n + 2) ** 2 * Fraction(1, 2**48)) * scale
        assert abs(got - exact) <= bound, (trial, n)
        if scale:
            worst = max(worst, float(abs(got - exact) / scale))
    # far below the bound in practice
    assert worst < 2.0**-44


def test_zero_weight_step_is_identity_for_finite_words():
    rng = np.random.default_rng(11)
    words = [0.0, -0.0, 1.0, -3.5, 3.4e38, -3.4e38, 1e-45, -1e-45, 1.1754944e-38, -2.5e-39]
    words += list(rng.normal(0, 1e3, 20))
    states = [(F(0.0), F(0.0))]
    for _ in range(30):
        n = int(rng.integers(1, 10))
        states.append(row_sum(rng.uniform(-1, 1, n), rng.lognormal(0, 3, n).astype(np.float32)))
    zero_hi, zero_lo = F(0.0), F(0.0)
    for h, l in states:
        for x in words:
            h2, l2 = ff_step(h, l, F(x), zero_hi, zero_lo)
            assert (bits(h2), bits(l2)) == (bits(h), bits(l)), (h, l, x)


def test_zero_weight_step_turns_non_finite_words_into_nan():
    h, l = row_sum([0.25, 0.5], np.array([3.0, 7.0], np.float32))
    for x in (np.inf, -np.inf, np.nan):
        h2, l2 = ff_step(h, l, F(x), F(0.0), F(0.0))
        assert np.isnan(h2) or np.isnan(l2)


def test_sums_never_reach_negative_zero():
    """The pair starts at +0 and a round-to-nearest sum is -0 only when both
    addends are -0, so h and l are never -0 (the padded steps' identity above
    needs it: -0 - (-0) would give +0)."""
    rng = np.random.default_rng(5)
    for _ in range(200):
        n = int(rng.integers(1, 8))
        ws = rng.choice([-1.0, 1.0], n) * rng.uniform(0, 1, n)
        xs = rng.choice([-1.0, 1.0, 0.0, -0.0], n).astype(np.float32)
        h, l = F(0.0), F(0.0)
        for w, x in zip(ws, xs):
            h, l = ff_step(h, l, x, *split(w))
            assert bits(h) != 0x80000000 and bits(l) != 0x80000000
