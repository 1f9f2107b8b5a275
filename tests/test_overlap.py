"""The float64 overlap reference used by the full-size gradient test, pinned
on the CPU: against exact rational arithmetic on random convex quads, and
against the upstream weights (golden fixture, 65^2 -> 49^2) where the
upstream's own sums are accurate."""

from fractions import Fraction

import numpy as np

import fixtures
from overlap import overlap_fraction


def _exact(qi, qo):
    def area(p):
        return sum(p[k][0] * p[(k + 1) % len(p)][1] - p[(k + 1) % len(p)][0] * p[k][1] for k in range(len(p))) / 2

    sgn = 1 if area(qi) > 0 else -1
    out = qo
    for k in range(4):
        a, b = qi[k], qi[(k + 1) % 4]
        if not out:
            break
        side = [sgn * ((b[0] - a[0]) * (p[1] - a[1]) - (b[1] - a[1]) * (p[0] - a[0])) for p in out]
        nxt = []
        for m, p in enumerate(out):
            q, sp, sq = out[(m + 1) % len(out)], side[m], side[(m + 1) % len(out)]
            if sp >= 0:
                nxt.append(p)
            if (sp >= 0) != (sq >= 0):
                t = sp / (sp - sq)
                nxt.append((p[0] + t * (q[0] - p[0]), p[1] + t * (q[1] - p[1])))
        out = nxt
    return abs(area(out)) / abs(area(qi)) if out else Fraction(0)


def test_overlap_against_exact_arithmetic():
    rng = np.random.default_rng(1)
    # a 3x3-cell input grid near (0.7, -0.4) with cells of ~2e-3 and a
    # jittered, slightly rotated output grid over it: many partial overlaps
    a = np.linspace(0, 6e-3, 4)
    x, y = np.meshgrid(a, a, indexing="ij")
    gi = (0.7 + x + 1e-4 * rng.normal(size=x.shape), -0.4 + y + 1e-4 * rng.normal(size=x.shape))
    b = np.linspace(-1e-3, 7e-3, 5)
    u, v = np.meshgrid(b, b, indexing="ij")
    c, s = np.cos(0.03), np.sin(0.03)
    go = (0.7 + c * u - s * v, -0.4 + s * u + c * v)
    ci, co = np.meshgrid(np.arange(9), np.arange(16), indexing="ij")
    ci, co = ci.ravel(), co.ravel()
    got = overlap_fraction(gi, go, ci, co)
    for k in range(ci.size):
        i, j = divmod(int(ci[k]), 3)
        m, n = divmod(int(co[k]), 4)
        qi = [(Fraction(gi[0][p, q]), Fraction(gi[1][p, q])) for p, q in ((i, j), (i + 1, j), (i + 1, j + 1), (i, j + 1))]
        qo = [(Fraction(go[0][p, q]), Fraction(go[1][p, q])) for p, q in ((m, n), (m + 1, n), (m + 1, n + 1), (m, n + 1))]
        assert abs(got[k] - float(_exact(qi, qo))) <= 1e-14, k
    assert np.sum(got > 0) > 20 and np.sum((got > 0) & (got < 1)) > 10


def test_overlap_against_upstream_weights():
    from regridding_gb300 import workloads

    c = fixtures.load("curvilinear.npz").case("curvi33")
    gi, go = c.tuple("ci"), workloads.perturb(c.tuple("co"))  # the fixture used the default jitter (seed 42)
    (ii, oo, vv), = c.weights()[0].reshape(-1)
    np.testing.assert_allclose(overlap_fraction(gi, go, ii, oo), vv, rtol=0, atol=1e-12)
