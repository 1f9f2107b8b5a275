"""Overlap fractions of quadrilateral cell pairs in float64, accurate to
about 1e-15 of the cell area: the output quad is clipped against the
(convex) input quad by Sutherland-Hodgman, with every coordinate taken
relative to the input quad's first vertex so that no product of absolute
coordinates cancels.  Test infrastructure: a reference for the geometry of
weights at sizes where the upstream's own sums (products of absolute
coordinates, `_weights_conservative_2d.py:752-830`) lose digits."""

import numpy as np


def _quads(x, y, cells, n1):
    i, j = np.divmod(np.asarray(cells, dtype=np.int64), n1)
    X = np.stack([x[i, j], x[i + 1, j], x[i + 1, j + 1], x[i, j + 1]], 1)
    Y = np.stack([y[i, j], y[i + 1, j], y[i + 1, j + 1], y[i, j + 1]], 1)
    return X, Y


def _shoelace(X, Y, n):
    m = X.shape[1]
    idx = np.arange(m)[None, :]
    valid = idx < n[:, None]
    nxt = np.where(idx + 1 < n[:, None], idx + 1, 0)
    X2 = np.take_along_axis(X, nxt, 1)
    Y2 = np.take_along_axis(Y, nxt, 1)
    return 0.5 * np.where(valid, X * Y2 - X2 * Y, 0.0).sum(1)


def overlap_fraction(grid_input, grid_output, cells_input, cells_output):
    """|input cell ∩ output cell| / |input cell| for each pair (flat cell
    indices, row-major over cells); input cells must be convex."""
    xi, yi = grid_input
    xo, yo = grid_output
    XI, YI = _quads(xi, yi, cells_input, xi.shape[1] - 1)
    PX, PY = _quads(xo, yo, cells_output, xo.shape[1] - 1)
    ox, oy = XI[:, :1].copy(), YI[:, :1].copy()
    XI, YI, PX, PY = XI - ox, YI - oy, PX - ox, PY - oy
    N = XI.shape[0]
    a_in = _shoelace(XI, YI, np.full(N, 4))
    sgn = np.sign(a_in)[:, None]
    M = 8  # two convex quads intersect in at most 8 vertices
    PX = np.concatenate([PX, np.zeros((N, M - 4))], 1)
    PY = np.concatenate([PY, np.zeros((N, M - 4))], 1)
    n = np.full(N, 4)
    idx = np.arange(M)[None, :]
    for k in range(4):
        ax, ay = XI[:, k:k + 1], YI[:, k:k + 1]
        bx, by = XI[:, (k + 1) % 4:(k + 1) % 4 + 1], YI[:, (k + 1) % 4:(k + 1) % 4 + 1]
        valid = idx < n[:, None]
        nxt = np.where(idx + 1 < n[:, None], idx + 1, 0)
        QX = np.take_along_axis(PX, nxt, 1)
        QY = np.take_along_axis(PY, nxt, 1)
        sp = sgn * ((bx - ax) * (PY - ay) - (by - ay) * (PX - ax))
        sq = sgn * ((bx - ax) * (QY - ay) - (by - ay) * (QX - ax))
        keep = valid & (sp >= 0)
        cross = valid & ((sp >= 0) != (sq >= 0))
        with np.errstate(all="ignore"):
            t = np.where(cross, sp / np.where(cross, sp - sq, 1.0), 0.0)
        IX = PX + t * (QX - PX)
        IY = PY + t * (QY - PY)
        CX = np.stack([PX, IX], 2).reshape(N, 2 * M)
        CY = np.stack([PY, IY], 2).reshape(N, 2 * M)
        CV = np.stack([keep, cross], 2).reshape(N, 2 * M)
        order = np.argsort(~CV, axis=1, kind="stable")
        PX = np.take_along_axis(CX, order, 1)[:, :M]
        PY = np.take_along_axis(CY, order, 1)[:, :M]
        n = np.minimum(CV.sum(1), M)
    return np.abs(_shoelace(PX, PY, n)) / np.abs(a_in)
