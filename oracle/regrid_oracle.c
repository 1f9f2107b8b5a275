/*
 * ORACLE — test infrastructure only.
 *
 * A plain-C restatement of the CPU loops of the upstream `regridding` package
 * (sun-data/regridding), used as the parity checker for the CUDA product and as
 * the timed CPU baseline.  Nothing in the product links or calls this file.
 *
 * Every routine follows the arithmetic of the upstream pure-Python execution
 * order exactly (the mode the upstream CI runs with NUMBA_DISABLE_JIT=1):
 * IEEE double, one rounding per Python operator, left-to-right evaluation,
 * no fused multiply-add.  Build with -ffp-contract=off (see Makefile) so that
 * results are bit-identical to the upstream pure-Python run; the golden
 * fixtures in tests/golden pin that.
 *
 * Citations are upstream paths relative to the project root.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAXSIZE INT64_MAX /* sys.maxsize on a 64-bit host */

/* status codes */
#define ORC_OK 0
#define ORC_ERR_ALLOC 1
#define ORC_ERR_WALK 2 /* a walk exceeded its step cap or was seated outside */

/* ------------------------------------------------------------------------- */
/* geometry primitives: regridding/geometry.py                               */
/* ------------------------------------------------------------------------- */

/* point_is_inside_box_2d: regridding/geometry.py:64-105 (inclusive bounds) */
static int inside_box(double x, double y, double x1, double y1, double x2, double y2) {
    if (!(x1 <= x && x <= x2)) return 0;
    if (!(y1 <= y && y <= y2)) return 0;
    return 1;
}

/* bounding_boxes_intersect_2d: regridding/geometry.py:153-284 */
static int bboxes_intersect(double xp1, double yp1, double xp2, double yp2,
                            double xq1, double yq1, double xq2, double yq2) {
    double t;
    if (xp1 > xp2) { t = xp1; xp1 = xp2; xp2 = t; }
    if (xq1 > xq2) { t = xq1; xq1 = xq2; xq2 = t; }
    if (!(xp1 <= xq2 && xq1 <= xp2)) return 0;
    if (yp1 > yp2) { t = yp1; yp1 = yp2; yp2 = t; }
    if (yq1 > yq2) { t = yq1; yq1 = yq2; yq2 = t; }
    if (!(yp1 <= yq2 && yq1 <= yp2)) return 0;
    return 1;
}

/* two_line_segment_intersection_parameters: regridding/geometry.py:370-445 */
static void seg_params(double x1, double y1, double x2, double y2,
                       double x3, double y3, double x4, double y4,
                       double *t, double *u) {
    if (!bboxes_intersect(x1, y1, x2, y2, x3, y3, x4, y4)) {
        *t = INFINITY;
        *u = INFINITY;
        return;
    }
    double tdet = (x1 - x3) * (y3 - y4) - (y1 - y3) * (x3 - x4);
    double udet = (x1 - x2) * (y1 - y3) - (y1 - y2) * (x1 - x3);
    double det = (x1 - x2) * (y3 - y4) - (y1 - y2) * (x3 - x4);
    *t = tdet / det;
    *u = -udet / det;
}

/* two_line_segments_intersect: regridding/geometry.py:448-475 (half-open) */
static int seg_hit(double t, double u) {
    return (0 <= t && t < 1) && (0 <= u && u < 1);
}

/* point_is_inside_polygon: regridding/geometry.py:737-829
 * (extended winding number with half crossings for vertices on the ray) */
static int inside_polygon(double x, double y, const double *vx, const double *vy,
                          int64_t n) {
    double w = 0;
    for (int64_t v = 0; v < n; v++) {
        int64_t i0 = (v == 0) ? n - 1 : v - 1;
        double x0 = vx[i0] - x;
        double y0 = vy[i0] - y;
        double x1 = vx[v] - x;
        double y1 = vy[v] - y;
        if (y0 * y1 < 0) {
            double r = x0 + y0 * (x1 - x0) / (y0 - y1);
            if (r > 0) {
                w += (y0 < 0) ? 1 : -1;
            } else {
                w += (y0 < 0) ? -1 : 1;
            }
        } else if (y0 == 0) {
            if (x0 > 0) {
                if (y1 > 0) w += 0.5;
                else if (y1 < 0) w -= 0.5;
            } else if (x0 < 0) {
                if (y1 < 0) w += 0.5;
                else if (y1 > 0) w -= 0.5;
            }
        } else if (y1 == 0) {
            if (x1 > 0) {
                if (y0 < 0) w += 0.5;
                else if (y0 > 0) w -= 0.5;
            } else if (x1 < 0) {
                if (y0 > 0) w += 0.5;
                else if (y0 < 0) w -= 0.5;
            }
        }
    }
    return w != 0;
}

/* ------------------------------------------------------------------------- */
/* grids: regridding/_weights/_weights_conservative_2d/_grids.py            */
/* ------------------------------------------------------------------------- */

typedef struct {
    const double *x, *y; /* row-major (nx, ny) vertex arrays */
    int64_t nx, ny;
} grid2;

static inline double gx(const grid2 *g, int64_t i, int64_t j) { return g->x[i * g->ny + j]; }
static inline double gy(const grid2 *g, int64_t i, int64_t j) { return g->y[i * g->ny + j]; }

/* grid_volume + _grid_volume_sweep: _grids.py:50-140.  The accumulation order
 * per cell is (((0 - a0[q]) + a0[q+1]) - a1[p]) + a1[p+1]. */
void orc_cell_area_2d(int64_t nx, int64_t ny, const double *x, const double *y, double *out) {
    int64_t ncx = nx - 1, ncy = ny - 1;
    for (int64_t k = 0; k < ncx * ncy; k++) out[k] = 0.0;
    /* axis 0: transposed and x/y swapped, so xa[i,j] = y[j,i], ya[i,j] = x[j,i];
     * num_i = ny, num_j = nx; out_aligned[i,j] = out[j,i] */
    for (int64_t j = 0; j < nx - 1; j++) {
        for (int64_t i = 0; i < ny; i++) {
            double x1 = y[j * ny + i], y1 = x[j * ny + i];
            double x2 = y[(j + 1) * ny + i], y2 = x[(j + 1) * ny + i];
            double area = (x1 * y2 - x2 * y1) / 2;
            if (i - 1 >= 0) out[j * ncy + (i - 1)] += area;
            if (i < ny - 1) out[j * ncy + i] -= area;
        }
    }
    /* axis 1: as stored */
    for (int64_t j = 0; j < ny - 1; j++) {
        for (int64_t i = 0; i < nx; i++) {
            double x1 = x[i * ny + j], y1 = y[i * ny + j];
            double x2 = x[i * ny + j + 1], y2 = y[i * ny + j + 1];
            double area = (x1 * y2 - x2 * y1) / 2;
            if (i - 1 >= 0) out[(i - 1) * ncy + j] += area;
            if (i < nx - 1) out[i * ncy + j] -= area;
        }
    }
}

/* grid_boundary: _grids.py:167-215 */
static void grid_boundary(const grid2 *g, double *bx, double *by) {
    int64_t n = 0, sx = g->nx, sy = g->ny;
    for (int64_t i = 0; i < sx - 1; i++, n++) { bx[n] = gx(g, i, 0); by[n] = gy(g, i, 0); }
    for (int64_t j = 0; j < sy - 1; j++, n++) { bx[n] = gx(g, sx - 1, j); by[n] = gy(g, sx - 1, j); }
    for (int64_t i = 0; i < sx - 1; i++, n++) { bx[n] = gx(g, sx - 1 - i, sy - 1); by[n] = gy(g, sx - 1 - i, sy - 1); }
    for (int64_t j = 0; j < sy - 1; j++, n++) { bx[n] = gx(g, 0, sy - 1 - j); by[n] = gy(g, 0, sy - 1 - j); }
}

static int cell_contains(const grid2 *g, int64_t i, int64_t j, double px, double py) {
    double vx[4], vy[4];
    vx[0] = gx(g, i, j);         vy[0] = gy(g, i, j);
    vx[1] = gx(g, i + 1, j);     vy[1] = gy(g, i + 1, j);
    vx[2] = gx(g, i + 1, j + 1); vy[2] = gy(g, i + 1, j + 1);
    vx[3] = gx(g, i, j + 1);     vy[3] = gy(g, i, j + 1);
    return inside_polygon(px, py, vx, vy, 4);
}

/* index_of_point_brute: _grids.py:218-279 */
void orc_locate_brute(const grid2 *g, double px, double py, int64_t *oi, int64_t *oj) {
    for (int64_t i = 0; i < g->nx - 1; i++)
        for (int64_t j = 0; j < g->ny - 1; j++)
            if (cell_contains(g, i, j, px, py)) { *oi = i; *oj = j; return; }
    *oi = ORC_MAXSIZE;
    *oj = ORC_MAXSIZE;
}

/* _index_of_point_local: _grids.py:282-349 */
static void locate_local(const grid2 *g, double px, double py, int64_t i0, int64_t j0,
                         int64_t *oi, int64_t *oj) {
    int64_t ncx = g->nx - 1, ncy = g->ny - 1;
    int64_t ia = i0 - 1 > 0 ? i0 - 1 : 0, ib = i0 + 2 < ncx ? i0 + 2 : ncx;
    int64_t ja = j0 - 1 > 0 ? j0 - 1 : 0, jb = j0 + 2 < ncy ? j0 + 2 : ncy;
    for (int64_t ii = ia; ii < ib; ii++)
        for (int64_t jj = ja; jj < jb; jj++)
            if (cell_contains(g, ii, jj, px, py)) { *oi = ii; *oj = jj; return; }
    *oi = ORC_MAXSIZE;
    *oj = ORC_MAXSIZE;
}

/* _bilinear_interpolation: regridding/_interp_ndarray.py:226-269 */
static double bilinear(const double *a, int64_t sx, int64_t sy, double x, double y) {
    int64_t x00 = (int64_t)floor(x), y00 = (int64_t)floor(y);
    if (x00 < 0) x00 = 0; else if (x00 > sx - 2) x00 = sx - 2;
    if (y00 < 0) y00 = 0; else if (y00 > sy - 2) y00 = sy - 2;
    double a00 = a[x00 * sy + y00], a01 = a[x00 * sy + y00 + 1];
    double a10 = a[(x00 + 1) * sy + y00], a11 = a[(x00 + 1) * sy + y00 + 1];
    double dx = x - (double)x00, dy = y - (double)y00;
    double w00 = (1 - dx) * (1 - dy), w01 = (1 - dx) * dy;
    double w10 = dx * (1 - dy), w11 = dx * dy;
    return (a00 * w00) + (a01 * w01) + (a10 * w10) + (a11 * w11);
}

/* A floor() that the upstream Python would reject (NaN, inf, beyond int64)
 * makes the iteration unusable; it is then resolved by the exhaustive search. */
static int floor_ok(double v) { return isfinite(v) && fabs(v) < 9.0e18; }

/* index_of_point_secant: _grids.py:352-463 */
void orc_locate_secant(const grid2 *g, double px, double py, int64_t *oi, int64_t *oj) {
    const double h = 1e-3;
    int64_t sx = g->nx, sy = g->ny;
    double i = (double)sx / 2, j = (double)sy / 2;
    for (int it = 0; it < 100; it++) {
        double xv = bilinear(g->x, sx, sy, i, j);
        double yv = bilinear(g->y, sx, sy, i, j);
        if (!floor_ok(i) || !floor_ok(j)) break;
        int64_t i0 = (int64_t)floor(i), j0 = (int64_t)floor(j);
        double ex = xv - px, ey = yv - py;
        if (i0 >= 0 && j0 >= 0 && i0 < sx - 1 && j0 < sy - 1) {
            if (cell_contains(g, i0, j0, px, py)) { locate_local(g, px, py, i0, j0, oi, oj); return; }
        }
        if (fabs(ex) < 1e-10 && fabs(ey) < 1e-10) { locate_local(g, px, py, i0, j0, oi, oj); return; }
        double dx_di = (bilinear(g->x, sx, sy, i + h, j) - xv) / h;
        double dx_dj = (bilinear(g->x, sx, sy, i, j + h) - xv) / h;
        double dy_di = (bilinear(g->y, sx, sy, i + h, j) - yv) / h;
        double dy_dj = (bilinear(g->y, sx, sy, i, j + h) - yv) / h;
        double det = dx_di * dy_dj - dx_dj * dy_di;
        if (det == 0) break;
        double di = (dy_dj * ex - dx_dj * ey) / det;
        double dj = (-dy_di * ex + dx_di * ey) / det;
        i -= di;
        j -= dj;
    }
    orc_locate_brute(g, px, py, oi, oj);
}

/* ------------------------------------------------------------------------- */
/* conservative 2D sweep:                                                     */
/* regridding/_weights/_weights_conservative_2d/_weights_conservative_2d.py  */
/* ------------------------------------------------------------------------- */

typedef struct {
    int64_t *in, *out;
    double *val;
    int64_t n, cap;
} tbuf;

static int tbuf_push(tbuf *b, int64_t i, int64_t o, double v) {
    if (b->n == b->cap) {
        int64_t nc = b->cap ? 2 * b->cap : 256;
        int64_t *ni = realloc(b->in, nc * sizeof(int64_t));
        if (!ni) return ORC_ERR_ALLOC;
        b->in = ni;
        int64_t *no = realloc(b->out, nc * sizeof(int64_t));
        if (!no) return ORC_ERR_ALLOC;
        b->out = no;
        double *nv = realloc(b->val, nc * sizeof(double));
        if (!nv) return ORC_ERR_ALLOC;
        b->val = nv;
        b->cap = nc;
    }
    b->in[b->n] = i;
    b->out[b->n] = o;
    b->val[b->n] = v;
    b->n++;
    return ORC_OK;
}

typedef struct {
    const grid2 *sweep;  /* unaligned sweep grid */
    int transposed;      /* axis_sweep == 0: aligned[a,b] = sweep[b,a] */
    int64_t sx, sy;      /* aligned shape */
    const grid2 *st;     /* static grid */
    int64_t ncx_st, ncy_st;
    const double *bx, *by; /* static boundary polygon */
    int64_t nb;
    double blx, bly, bux, buy; /* static bbox */
    const double *area_in;
    const double *w_in; /* may be NULL */
    int64_t ncx_in, ncy_in, ncx_out, ncy_out;
    int sweep_input, axis;
} sweep_ctx;

static inline double swx(const sweep_ctx *c, int64_t a, int64_t b) {
    return c->transposed ? gx(c->sweep, b, a) : gx(c->sweep, a, b);
}
static inline double swy(const sweep_ctx *c, int64_t a, int64_t b) {
    return c->transposed ? gy(c->sweep, b, a) : gy(c->sweep, a, b);
}

/* _calc_and_save_weights + _index_input_output: :898-1058 */
static int save_weights(const sweep_ctx *c, double x1, double y1, double x2, double y2,
                        int64_t i, int64_t j, int64_t stx, int64_t sty, tbuf *b) {
    double area = (x1 * y2 - x2 * y1) / 2;
    if (c->axis == 0) area = -area;
    for (int side = 0; side < 2; side++) {
        int64_t is = side == 0 ? i - 1 : i;
        if (side == 0 && !(is >= 0)) continue;
        if (side == 1 && !(is < c->sx - 1)) continue;
        int64_t a = is, bb = j;
        if (c->axis == 0) { a = j; bb = is; }
        int64_t ii, ij, oi, oj;
        if (c->sweep_input) { ii = a; ij = bb; oi = stx; oj = sty; }
        else { ii = stx; ij = sty; oi = a; oj = bb; }
        double ain = c->area_in[ii * c->ncy_in + ij];
        double w = side == 0 ? area / ain : -area / ain;
        if (c->w_in) w = w * c->w_in[ii * c->ncy_in + ij];
        int rc = tbuf_push(b, ii * c->ncy_in + ij, oi * c->ncy_out + oj, w);
        if (rc) return rc;
    }
    return ORC_OK;
}

static const int vtx_i[4] = {0, 1, 1, 0}; /* indices_cell_vertex: _grids.py:153-158 */
static const int vtx_j[4] = {0, 0, 1, 1};
static const int nrm_i[4] = {-1, 0, 1, 0}; /* cell_normals: _grids.py:143-148 */
static const int nrm_j[4] = {0, -1, 0, 1};

/* one sweep line: the body of the prange loop of _sweep_along_axis,
 * :432-533, with _step_outside_static (:547-698) and _step_inside_static
 * (:707-895) inlined. */
static int sweep_line(const sweep_ctx *c, int64_t line, int64_t max_steps, tbuf *b) {
    const grid2 *st = c->st;
    int64_t sy_idx = 0;
    int64_t stx = ORC_MAXSIZE, sty = ORC_MAXSIZE;
    int outside = 1;
    int64_t edge_last = ORC_MAXSIZE;
    double x1 = swx(c, line, 0), y1 = swy(c, line, 0);
    if (inside_box(x1, y1, c->blx, c->bly, c->bux, c->buy)) {
        if (inside_polygon(x1, y1, c->bx, c->by, c->nb)) {
            orc_locate_secant(st, x1, y1, &stx, &sty);
            outside = 0;
            if (stx == ORC_MAXSIZE) return ORC_ERR_WALK; /* upstream indexes out of range here */
        }
    }
    int64_t steps = 0;
    while (sy_idx < c->sy - 1) {
        if (++steps > max_steps) return ORC_ERR_WALK;
        double x2 = swx(c, line, sy_idx + 1), y2 = swy(c, line, sy_idx + 1);
        if (outside) {
            /* _step_outside_static */
            double p2x = x2, p2y = y2;
            int64_t new_edge_last = ORC_MAXSIZE;
            int found = 0;
            double t_min = INFINITY;
            for (int axis = 0; axis < 2; axis++) {
                int64_t num_i = axis == 0 ? st->ny : st->nx;
                for (int dir = 0; dir < 2; dir++) {
                    for (int64_t i0 = 0; i0 < num_i - 1; i0++) {
                        double x3, y3, x4, y4;
                        if (axis == 0) {
                            int64_t ie = dir ? st->nx - 1 : 0;
                            x3 = gx(st, ie, i0); y3 = gy(st, ie, i0);
                            x4 = gx(st, ie, i0 + 1); y4 = gy(st, ie, i0 + 1);
                        } else {
                            int64_t je = dir ? st->ny - 1 : 0;
                            x3 = gx(st, i0, je); y3 = gy(st, i0, je);
                            x4 = gx(st, i0 + 1, je); y4 = gy(st, i0 + 1, je);
                        }
                        double t, u;
                        seg_params(x1, y1, p2x, p2y, x3, y3, x4, y4, &t, &u);
                        if (seg_hit(t, u) && t < t_min) {
                            int64_t n = dir ? (axis == 0 ? c->ncx_st : c->ncy_st) - 1 : 0;
                            int64_t cx = axis == 0 ? n : i0, cy = axis == 0 ? i0 : n;
                            if (cx * c->ncy_st + cy == edge_last) continue;
                            found = 1;
                            t_min = t;
                            stx = cx;
                            sty = cy;
                            x2 = x1 + t * (p2x - x1);
                            y2 = y1 + t * (p2y - y1);
                            new_edge_last = dir * 2 + axis;
                            outside = 0;
                        }
                    }
                }
            }
            edge_last = new_edge_last;
            if (!found) sy_idx = sy_idx + 1;
        } else {
            /* _step_inside_static */
            double p2x = x2, p2y = y2;
            int found = -1;
            for (int v = 0; v < 4; v++) {
                if (v == edge_last) continue;
                int vp = (v + 3) & 3;
                double x3 = gx(st, stx + vtx_i[vp], sty + vtx_j[vp]);
                double y3 = gy(st, stx + vtx_i[vp], sty + vtx_j[vp]);
                double x4 = gx(st, stx + vtx_i[v], sty + vtx_j[v]);
                double y4 = gy(st, stx + vtx_i[v], sty + vtx_j[v]);
                double t, u;
                seg_params(x1, y1, p2x, p2y, x3, y3, x4, y4, &t, &u);
                if (seg_hit(t, u)) {
                    x2 = x1 + t * (p2x - x1);
                    y2 = y1 + t * (p2y - y1);
                    found = v;
                    break;
                }
            }
            int64_t nsy, nstx, nsty;
            if (found >= 0) {
                nsy = sy_idx;
                nstx = stx + nrm_i[found];
                nsty = sty + nrm_j[found];
                edge_last = (found + 2) % 4;
            } else {
                nsy = sy_idx + 1;
                nstx = stx;
                nsty = sty;
                edge_last = ORC_MAXSIZE;
            }
            int rc = save_weights(c, x1, y1, x2, y2, line, sy_idx, stx, sty, b);
            if (rc) return rc;
            if (!(nstx >= 0 && nsty >= 0 && nstx < c->ncx_st && nsty < c->ncy_st)) {
                edge_last = stx * c->ncy_st + sty;
                nstx = ORC_MAXSIZE;
                nsty = ORC_MAXSIZE;
                outside = 1;
            }
            sy_idx = nsy;
            stx = nstx;
            sty = nsty;
        }
        x1 = x2;
        y1 = y2;
    }
    return ORC_OK;
}

/* Result of a sweep: raw triples in the upstream emission order
 * (_compact_rows, :27-73). Freed with orc_free. */
typedef struct {
    int64_t n;
    int64_t *in, *out;
    double *val;
} orc_triples;

void orc_free(void *p) { free(p); }

/* weights_conservative_2d: :80-126.  Grids are contiguous (nx, ny) arrays.
 * w_in is NULL or a (ncx_in, ncy_in) array.  On success the three arrays in
 * *res are malloc'd and owned by the caller (orc_free). */
int orc_sweep_2d(int64_t nxi, int64_t nyi, const double *xi, const double *yi,
                 int64_t nxo, int64_t nyo, const double *xo, const double *yo,
                 const double *w_in, int nthreads, orc_triples *res) {
    grid2 gin = {xi, yi, nxi, nyi}, gout = {xo, yo, nxo, nyo};
    int64_t ncx_in = nxi - 1, ncy_in = nyi - 1;
    double *area_in = malloc(sizeof(double) * (size_t)(ncx_in * ncy_in > 0 ? ncx_in * ncy_in : 1));
    if (!area_in) return ORC_ERR_ALLOC;
    orc_cell_area_2d(nxi, nyi, xi, yi, area_in);

    int64_t nlines_total = 2 * nxo + 2 * nyo + 2 * nxi + 2 * nyi;
    tbuf *bufs = calloc((size_t)nlines_total, sizeof(tbuf));
    if (!bufs) { free(area_in); return ORC_ERR_ALLOC; }
    int status = ORC_OK;
    int64_t base = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    for (int sweep_input = 0; sweep_input < 2; sweep_input++) {
        const grid2 *gs = sweep_input ? &gin : &gout;
        const grid2 *gt = sweep_input ? &gout : &gin;
        int64_t nb = 2 * (gt->nx - 1) + 2 * (gt->ny - 1);
        double *bx = malloc(sizeof(double) * (size_t)nb), *by = malloc(sizeof(double) * (size_t)nb);
        if (!bx || !by) { free(bx); free(by); status = ORC_ERR_ALLOC; break; }
        grid_boundary(gt, bx, by);
        double blx = gt->x[0], bly = gt->y[0], bux = gt->x[0], buy = gt->y[0];
        for (int64_t k = 0; k < gt->nx * gt->ny; k++) {
            /* ndarray.min/max: NaN propagates; grids here are finite */
            if (gt->x[k] < blx) blx = gt->x[k];
            if (gt->x[k] > bux) bux = gt->x[k];
            if (gt->y[k] < bly) bly = gt->y[k];
            if (gt->y[k] > buy) buy = gt->y[k];
        }
        for (int axis = 0; axis < 2; axis++) {
            sweep_ctx c;
            c.sweep = gs;
            c.transposed = axis == 0;
            c.sx = axis == 0 ? gs->ny : gs->nx;
            c.sy = axis == 0 ? gs->nx : gs->ny;
            c.st = gt;
            c.ncx_st = gt->nx - 1;
            c.ncy_st = gt->ny - 1;
            c.bx = bx; c.by = by; c.nb = nb;
            c.blx = blx; c.bly = bly; c.bux = bux; c.buy = buy;
            c.area_in = area_in;
            c.w_in = w_in;
            c.ncx_in = ncx_in; c.ncy_in = ncy_in;
            c.ncx_out = nxo - 1; c.ncy_out = nyo - 1;
            c.sweep_input = sweep_input;
            c.axis = axis;
            int64_t max_steps = 64 * (c.sy + 4 * (c.ncx_st + c.ncy_st) + 16);
            int local_status = ORC_OK;
#pragma omp parallel for schedule(dynamic, 1)
            for (int64_t line = 0; line < c.sx; line++) {
                int rc = sweep_line(&c, line, max_steps, &bufs[base + line]);
                if (rc) {
#pragma omp critical
                    local_status = rc;
                }
            }
            if (local_status) status = local_status;
            base += c.sx;
        }
        free(bx);
        free(by);
        if (status) break;
    }
    int64_t total = 0;
    for (int64_t k = 0; k < base; k++) total += bufs[k].n;
    res->n = total;
    res->in = malloc(sizeof(int64_t) * (size_t)(total > 0 ? total : 1));
    res->out = malloc(sizeof(int64_t) * (size_t)(total > 0 ? total : 1));
    res->val = malloc(sizeof(double) * (size_t)(total > 0 ? total : 1));
    if (!res->in || !res->out || !res->val) status = status ? status : ORC_ERR_ALLOC;
    int64_t w = 0;
    for (int64_t k = 0; k < nlines_total; k++) {
        if (!status) {
            memcpy(res->in + w, bufs[k].in, sizeof(int64_t) * (size_t)bufs[k].n);
            memcpy(res->out + w, bufs[k].out, sizeof(int64_t) * (size_t)bufs[k].n);
            memcpy(res->val + w, bufs[k].val, sizeof(double) * (size_t)bufs[k].n);
            w += bufs[k].n;
        }
        free(bufs[k].in);
        free(bufs[k].out);
        free(bufs[k].val);
    }
    free(bufs);
    free(area_in);
    return status;
}

/* locate many points (brute or secant) on one grid */
void orc_locate_many(int64_t nx, int64_t ny, const double *x, const double *y, int64_t n,
                     const double *px, const double *py, int method, int64_t *oi, int64_t *oj) {
    grid2 g = {x, y, nx, ny};
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t k = 0; k < n; k++) {
        if (method == 0) orc_locate_brute(&g, px[k], py[k], &oi[k], &oj[k]);
        else orc_locate_secant(&g, px[k], py[k], &oi[k], &oj[k]);
    }
}

/* ------------------------------------------------------------------------- */
/* apply: regridding/_regrid/_regrid_from_weights.py:165-182                 */
/* values_output[d, o] += w * values_input[d, i], entries in stored order.  */
/* The f32-input variant promotes each value to double, as numpy does.       */
/* ------------------------------------------------------------------------- */
void orc_apply_f64(int64_t ndim_d, int64_t n_in, int64_t n_out, int64_t nnz,
                   const int64_t *ii, const int64_t *oo, const double *w,
                   const double *vin, double *vout) {
#pragma omp parallel for schedule(static)
    for (int64_t d = 0; d < ndim_d; d++) {
        const double *a = vin + d * n_in;
        double *b = vout + d * n_out;
        for (int64_t k = 0; k < n_out; k++) b[k] = 0.0;
        for (int64_t k = 0; k < nnz; k++) {
            int64_t i = ii[k] < 0 ? ii[k] + n_in : ii[k];
            int64_t o = oo[k] < 0 ? oo[k] + n_out : oo[k];
            b[o] = b[o] + w[k] * a[i];
        }
    }
}

void orc_apply_f32in(int64_t ndim_d, int64_t n_in, int64_t n_out, int64_t nnz,
                     const int64_t *ii, const int64_t *oo, const double *w,
                     const float *vin, double *vout) {
#pragma omp parallel for schedule(static)
    for (int64_t d = 0; d < ndim_d; d++) {
        const float *a = vin + d * n_in;
        double *b = vout + d * n_out;
        for (int64_t k = 0; k < n_out; k++) b[k] = 0.0;
        for (int64_t k = 0; k < nnz; k++) {
            int64_t i = ii[k] < 0 ? ii[k] + n_in : ii[k];
            int64_t o = oo[k] < 0 ? oo[k] + n_out : oo[k];
            b[o] = b[o] + w[k] * (double)a[i];
        }
    }
}

/* f32 output given in place (values_output of dtype float32): each update is
 * computed in double and stored back rounded to float, as numpy does. */
void orc_apply_f32in_f32out(int64_t ndim_d, int64_t n_in, int64_t n_out, int64_t nnz,
                            const int64_t *ii, const int64_t *oo, const double *w,
                            const float *vin, float *vout) {
#pragma omp parallel for schedule(static)
    for (int64_t d = 0; d < ndim_d; d++) {
        const float *a = vin + d * n_in;
        float *b = vout + d * n_out;
        for (int64_t k = 0; k < n_out; k++) b[k] = 0.0f;
        for (int64_t k = 0; k < nnz; k++) {
            int64_t i = ii[k] < 0 ? ii[k] + n_in : ii[k];
            int64_t o = oo[k] < 0 ? oo[k] + n_out : oo[k];
            b[o] = (float)((double)b[o] + w[k] * (double)a[i]);
        }
    }
}

/* ------------------------------------------------------------------------- */
/* find_indices 1D                                                            */
/* ------------------------------------------------------------------------- */

/* numpy.searchsorted(a, v, side="left") for an ascending a: first k with
 * a[k] >= v, NaN sorting last. */
static int64_t lower_bound_np(const double *a, int64_t n, double v) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = lo + ((hi - lo) >> 1);
        double am = a[mid];
        /* numpy's less-than for floats: a < b, or b is NaN and a is not */
        int lt = (am < v) || (isnan(v) && !isnan(am));
        if (lt) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

/* _find_indices_searchsorted_1d: _find_indices_searchsorted.py:24-62 */
void orc_find_indices_searchsorted(int64_t nd, int64_t m, const double *xin, int64_t xin_stride,
                                   int64_t n, const double *xout, int64_t xout_stride,
                                   int64_t fill, int64_t *res) {
#pragma omp parallel for schedule(static)
    for (int64_t d = 0; d < nd; d++) {
        const double *a = xin + d * xin_stride;
        const double *p = xout + d * xout_stride;
        for (int64_t i = 0; i < n; i++) {
            int64_t r = lower_bound_np(a, m, p[i]) - 1;
            if (p[i] == a[0]) r = 0;
            else if (r < 0) r = fill;
            else if (r > m - 2) r = fill;
            res[d * n + i] = r;
        }
    }
}

/* _find_indices_brute_1d: _find_indices_brute.py:24-51 */
void orc_find_indices_brute(int64_t nd, int64_t m, const double *xin, int64_t xin_stride,
                            int64_t n, const double *xout, int64_t xout_stride,
                            int64_t fill, int64_t *res) {
#pragma omp parallel for schedule(static)
    for (int64_t d = 0; d < nd; d++) {
        const double *a = xin + d * xin_stride;
        const double *p = xout + d * xout_stride;
        for (int64_t i = 0; i < n; i++) {
            int64_t r = fill;
            for (int64_t k = 0; k < m - 1; k++) {
                if (a[k] <= p[i] && p[i] <= a[k + 1]) { r = k; break; }
            }
            res[d * n + i] = r;
        }
    }
}

/* _weights_from_indices_multilinear_1d: _weights_multilinear.py:142-206.
 * idx holds already-resolved cells (clamped, side recovered, :115-119). */
void orc_multilinear_1d(int64_t nd, int64_t m, const double *xin, int64_t xin_stride,
                        int64_t n, const double *xout, int64_t xout_stride,
                        const int64_t *idx, const double *w_in, int64_t w_in_stride,
                        const uint8_t *outside, int64_t *ind_in, int64_t *ind_out,
                        double *val) {
    (void)m;
#pragma omp parallel for schedule(static)
    for (int64_t d = 0; d < nd; d++) {
        const double *a = xin + d * xin_stride;
        const double *p = xout + d * xout_stride;
        for (int64_t i = 0; i < n; i++) {
            int64_t i0 = idx[d * n + i], i1 = i0 + 1;
            double x0 = a[i0], x1 = a[i1], x = p[i];
            double w1 = (x - x0) / (x1 - x0);
            double w0 = 1 - w1;
            if (w_in) {
                w0 = w0 * w_in[d * w_in_stride + i0];
                w1 = w1 * w_in[d * w_in_stride + i1];
            }
            if (outside && outside[d * n + i]) { w0 = NAN; w1 = NAN; }
            int64_t k = d * 2 * n + 2 * i;
            ind_in[k] = i0; ind_out[k] = i; val[k] = w0;
            ind_in[k + 1] = i1; ind_out[k + 1] = i; val[k + 1] = w1;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* conservative 1D: regridding/_weights/_weights_conservative_1d/ (all files) */
/* ------------------------------------------------------------------------- */

/* index_of_point: _weights_conservative_1d/_grids.py:38-73 */
static int64_t index_of_point_1d(double p, const double *g, int64_t n) {
    int64_t l = 0, r = n;
    while (r - l > 1) {
        int64_t mid = (l + r) / 2;
        if (g[mid] > p) r = mid;
        else l = mid;
    }
    return r;
}

/* _weights_conservative_1d: _weights_conservative_1d.py:59-318.  Writes at most
 * cap triples; returns the count (or -1 if cap is too small). */
int64_t orc_conservative_1d(int64_t nin, const double *xin_raw, int64_t nout, const double *xout_raw,
                            const double *w_in, int64_t cap, int64_t *ind_in, int64_t *ind_out,
                            double *val, double *work) {
    /* work: nin + nout + (nin - 1) doubles */
    double *xs = work, *xt = work + nin, *len_in = work + nin + nout;
    int rev_in = !(xin_raw[0] < xin_raw[nin - 1]);
    int rev_out = !(xout_raw[0] < xout_raw[nout - 1]);
    for (int64_t k = 0; k < nin; k++) xs[k] = rev_in ? xin_raw[nin - 1 - k] : xin_raw[k];
    for (int64_t k = 0; k < nout; k++) xt[k] = rev_out ? xout_raw[nout - 1 - k] : xout_raw[k];
    double st_left = xt[0], st_right = xt[nout - 1];
    for (int64_t k = 0; k < nin - 1; k++) len_in[k] = xs[k + 1] - xs[k];
    int64_t isw = 0, ist, count = 0;
    double p1 = xs[0];
    int outside;
    if (st_left == p1) { outside = 0; ist = 0; }
    else if (st_left < p1 && p1 < st_right) { outside = 0; ist = index_of_point_1d(p1, xt, nout) - 1; }
    else { outside = 1; ist = ORC_MAXSIZE; }
    while (isw < nin - 1) {
        double p2 = xs[isw + 1];
        if (outside) {
            /* _step_outside_static: :192-236 */
            double ps = xt[0];
            if (p1 < ps && ps < p2) { ist = 0; p2 = ps; }
            else if (ps == p2) { isw = isw + 1; ist = 0; }
            else { isw = isw + 1; }
            if (ist < ORC_MAXSIZE) outside = 0;
        } else {
            /* _step_inside_static: :239-318 */
            int64_t iin = isw, iout = ist;
            if (rev_in) iin = ~iin;
            if (rev_out) iout = ~iout;
            double ps = xt[ist + 1];
            if (p1 < ps && ps < p2) { ist = ist + 1; p2 = ps; }
            else if (ps == p2) { ist = ist + 1; isw = isw + 1; }
            else { isw = isw + 1; }
            double length = p2 - p1;
            /* Python negative indexing into the (reversed-grid) length array */
            int64_t li = iin < 0 ? iin + (nin - 1) : iin;
            double ratio = length / len_in[li];
            if (w_in) {
                int64_t wi = iin < 0 ? iin + (nin - 1) : iin;
                ratio = ratio * w_in[wi];
            }
            if (count >= cap) return -1;
            ind_in[count] = iin; ind_out[count] = iout; val[count] = ratio;
            count++;
            if (!(0 <= ist && ist < nout - 1)) break;
        }
        p1 = p2;
    }
    return count;
}

/* ------------------------------------------------------------------------
 * Red-black Gauss-Seidel fill: _fill_gauss_seidel_2d and
 * _iteration_gauss_seidel_2d (regridding/_fill/_gauss_seidel.py:83-139).
 * a is (nt, ny, nx) C-ordered; only cells with where != 0 are rewritten.
 * The float64 loop keeps the sequential sweep order (j outer, i inner) and
 * the periodic neighbours; every operation rounds once.
 * ------------------------------------------------------------------------ */
static void gs_constants(int64_t nx, int64_t ny, double *dxxinv, double *dyyinv, double *dcent) {
    const double dx = 2.0 / (double)(nx - 1);
    const double dy = 2.0 / (double)(ny - 1);
    *dxxinv = 1.0 / (dx * dx);
    *dyyinv = 1.0 / (dy * dy);
    *dcent = 1.0 / (2.0 * (*dxxinv + *dyyinv));
}

void orc_fill_gauss_seidel_f64(int64_t nt, int64_t ny, int64_t nx, double *a, const uint8_t *where,
                               int64_t iterations) {
    double dxxinv, dyyinv, dcent;
    gs_constants(nx, ny, &dxxinv, &dyyinv, &dcent);
    for (int64_t t = 0; t < nt; ++t) {
        double *s = a + t * ny * nx;
        const uint8_t *w = where + t * ny * nx;
        for (int64_t k = 0; k < iterations; ++k) {
            for (int64_t odd = 0; odd < 2; ++odd) {
                for (int64_t j = 0; j < ny; ++j) {
                    for (int64_t i = 0; i < nx; ++i) {
                        if (((i + j) & 1) != odd || !w[j * nx + i]) continue;
                        const int64_t i9 = (i - 1 + nx) % nx, i1 = (i + 1) % nx;
                        const int64_t j9 = (j - 1 + ny) % ny, j1 = (j + 1) % ny;
                        const double xterm = dxxinv * (s[j * nx + i9] + s[j * nx + i1]);
                        const double yterm = dyyinv * (s[j9 * nx + i] + s[j1 * nx + i]);
                        s[j * nx + i] = (xterm + yterm) * dcent;
                    }
                }
            }
        }
    }
}

/* float32 arrays under Numba's typing: the neighbour sums are float32, the
 * products with the float64 constants and the rest are float64, and the
 * stored value is rounded to float32. */
void orc_fill_gauss_seidel_f32(int64_t nt, int64_t ny, int64_t nx, float *a, const uint8_t *where,
                               int64_t iterations) {
    double dxxinv, dyyinv, dcent;
    gs_constants(nx, ny, &dxxinv, &dyyinv, &dcent);
    for (int64_t t = 0; t < nt; ++t) {
        float *s = a + t * ny * nx;
        const uint8_t *w = where + t * ny * nx;
        for (int64_t k = 0; k < iterations; ++k) {
            for (int64_t odd = 0; odd < 2; ++odd) {
                for (int64_t j = 0; j < ny; ++j) {
                    for (int64_t i = 0; i < nx; ++i) {
                        if (((i + j) & 1) != odd || !w[j * nx + i]) continue;
                        const int64_t i9 = (i - 1 + nx) % nx, i1 = (i + 1) % nx;
                        const int64_t j9 = (j - 1 + ny) % ny, j1 = (j + 1) % ny;
                        const float sx = s[j * nx + i9] + s[j * nx + i1];
                        const float sy = s[j9 * nx + i] + s[j1 * nx + i];
                        const double xterm = dxxinv * (double)sx;
                        const double yterm = dyyinv * (double)sy;
                        s[j * nx + i] = (float)((xterm + yterm) * dcent);
                    }
                }
            }
        }
    }
}
