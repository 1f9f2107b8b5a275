// Conservative 2D weights on the GPU: the Ramshaw (1985) edge sweep.
//
// Every grid line of the output grid is traced through the cells of the input
// grid and every grid line of the input grid through the cells of the output
// grid.  Each piece of a line inside one cell of the other grid contributes
// the contour integral 1/2 (x1 y2 - x2 y1) to the two cells of its own grid
// that it separates (Green's theorem); the contributions of one
// (input, output) pair sum to their overlap area.
//
// The walk follows regridding/_weights/_weights_conservative_2d/
// _weights_conservative_2d.py:206-912 step for step with the same IEEE double
// arithmetic (one rounding per operation, no FMA), so crossing decisions,
// emitted triples and their order are identical to the upstream code.  What
// is GB300-specific is the organisation:
//   * seat kernel: one warp per sweep line computes the line's starting state
//     (the O(perimeter) winding-number test is split across the lanes; its
//     partial sums are multiples of 1/2 and therefore exact in any order);
//   * walk kernel: one thread per sweep line, run twice (count, then write at
//     scanned offsets), which reproduces the upstream emission order without
//     a sort on sequence numbers;
//   * the O(perimeter) search for re-entry into the static grid
//     (_step_outside_static, :547-698) is answered from a uniform bin grid of
//     the static boundary, evaluating exactly the candidate edges whose
//     bounding boxes can pass the upstream box test and keeping the upstream
//     "first smallest t" choice;
//   * merge: raw triples are bucketed by output cell, ranked by (input,
//     emission position) inside each bucket, and equal pairs are summed with
//     numpy's add.reduceat association (first + pairwise rest), giving a CSR
//     matrix whose values are bit-identical to the upstream coalesced ones.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "seed.cuh"

namespace rg {
namespace {

// ---------------------------------------------------------------------------
// geometry (regridding/geometry.py)
// ---------------------------------------------------------------------------

// Order-preserving integer image of a double for the comparisons below:
// keys compare (signed) as the doubles do, -0.0 and +0.0 share a key, and
// NaN is handled by the caller.  Integer compares keep the walk's many
// bounding-box tests off the FP64 pipe (2 lanes per clock per SM on GB300).
__device__ __forceinline__ long long order_key(double v) {
    const long long b = __double_as_longlong(v);
    if ((b & 0x7fffffffffffffffll) == 0) return 0;
    return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}

__device__ __forceinline__ bool any_nan(double a, double b, double c, double d) {
    const unsigned long long m = 0x7fffffffffffffffull, inf = 0x7ff0000000000000ull;
    return (((unsigned long long)__double_as_longlong(a) & m) > inf) |
           (((unsigned long long)__double_as_longlong(b) & m) > inf) |
           (((unsigned long long)__double_as_longlong(c) & m) > inf) |
           (((unsigned long long)__double_as_longlong(d) & m) > inf);
}

// bounding_boxes_intersect_2d: geometry.py:153-284.  The upstream orders
// each pair and compares min/max; any NaN coordinate makes one of its
// comparisons false, so NaN means no intersection here too.
__device__ __forceinline__ bool bboxes_intersect(double xp1, double yp1, double xp2, double yp2,
                                                 double xq1, double yq1, double xq2, double yq2) {
    if (any_nan(xp1, xp2, xq1, xq2) || any_nan(yp1, yp2, yq1, yq2)) return false;
    long long a = order_key(xp1), b = order_key(xp2), c = order_key(xq1), d = order_key(xq2);
    if (!(min(a, b) <= max(c, d) && min(c, d) <= max(a, b))) return false;
    a = order_key(yp1), b = order_key(yp2), c = order_key(yq1), d = order_key(yq2);
    return min(a, b) <= max(c, d) && min(c, d) <= max(a, b);
}

// two_line_segment_intersection_parameters (geometry.py:370-445) followed by
// two_line_segments_intersect (geometry.py:448-475, half-open 0 <= t,u < 1).
// True only when the rounded quotient fl(n / d) is certainly outside [0, 1),
// decided on the bits without dividing (integer operations; GB300 runs FP64
// at 2 lanes per clock per SM and a division is about ten FP64 operations).
// For |d| < 2^52 (finite):
//   d == 0                  -> n / d is +-inf or NaN;
//   |n| >= |d|              -> |n / d| >= 1, rounds to a magnitude >= 1;
//   n, d of opposite signs  -> n / d < 0, and with |n| >= 2^-1022 its
//                              magnitude exceeds 2^-1075, so it rounds to a
//                              negative number, not to -0.
// Anything else returns false and the caller divides, so the test it
// guards gives the same answer as dividing every time.
__device__ __forceinline__ bool quotient_outside_unit(double n, double d) {
    const unsigned long long abs_mask = 0x7fffffffffffffffull;
    const unsigned long long nb = (unsigned long long)__double_as_longlong(n);
    const unsigned long long db = (unsigned long long)__double_as_longlong(d);
    const unsigned long long na = nb & abs_mask, da = db & abs_mask;
    if (da >= 0x4330000000000000ull) return false;  // |d| >= 2^52, inf or NaN: divide
    if (da == 0 || na >= da) return true;
    return na >= 0x0010000000000000ull && ((nb ^ db) >> 63);
}

// Where the rounded quotient fl(n / d) lies against [0, 1), decided on the
// bits when that is certain: 0 outside, 1 inside, -1 undecided (divide).
// Inside is certain for n == 0, or n and d of one sign with |n| at least two
// representable steps below |d|: then n / d <= 1 - 2^-52, which rounds
// below 1.  Outside follows quotient_outside_unit.  A NaN n is undecided.
__device__ __forceinline__ int quotient_in_unit(double n, double d) {
    const unsigned long long abs_mask = 0x7fffffffffffffffull;
    const unsigned long long nb = (unsigned long long)__double_as_longlong(n);
    const unsigned long long db = (unsigned long long)__double_as_longlong(d);
    const unsigned long long na = nb & abs_mask, da = db & abs_mask;
    if (da >= 0x4330000000000000ull || na > 0x7ff0000000000000ull) return -1;
    if (da == 0 || na >= da) return 0;
    if (na == 0) return 1;
    if ((nb ^ db) >> 63) return na >= 0x0010000000000000ull ? 0 : -1;
    return na + 2 <= da ? 1 : -1;
}

__device__ __forceinline__ bool seg_hit(double x1, double y1, double x2, double y2, double x3,
                                        double y3, double x4, double y4, double* t_out) {
    if (!bboxes_intersect(x1, y1, x2, y2, x3, y3, x4, y4)) return false;
    double tdet = dsub(dmul(dsub(x1, x3), dsub(y3, y4)), dmul(dsub(y1, y3), dsub(x3, x4)));
    double udet = dsub(dmul(dsub(x1, x2), dsub(y1, y3)), dmul(dsub(y1, y2), dsub(x1, x3)));
    double det = dsub(dmul(dsub(x1, x2), dsub(y3, y4)), dmul(dsub(y1, y2), dsub(x3, x4)));
    // most candidate edges miss: reject them before the two divisions
    if (quotient_outside_unit(tdet, det) || quotient_outside_unit(-udet, det)) return false;
    double t = ddiv(tdet, det);
    double u = ddiv(-udet, det);
    *t_out = t;
    return (0 <= t && t < 1) && (0 <= u && u < 1);
}

// ---------------------------------------------------------------------------
// Certified float32 filter for the walk's crossing test.  On GB300 the FP64
// pipe runs 2 lanes per clock per SM (1/64 of FP32), and the 13 FP64
// operations of each candidate edge's determinants were over half of the
// walk.  The filter evaluates the same determinants in float32 from
// coordinates truncated to float32 (from their bits: no FP64 instruction),
// with a static error bound in the manner of Shewchuk's adaptive predicates
// (Shewchuk 1997, "Adaptive precision floating-point arithmetic and fast
// robust geometric predicates"), and answers only where the FP64 result is
// certain; the walk computes the FP64 determinants of the edge it crosses
// (its t is needed) and of the rare undecided candidates.
// ---------------------------------------------------------------------------

// v truncated to float32 from its bits: |v - f| < 2^-23 |v|.  Magnitudes
// below 2^-126 give 0; magnitudes of 2^128 or more (and inf, NaN) clear ok.
__device__ __forceinline__ float trunc_float(double v, bool& ok) {
    const unsigned hi = (unsigned)__double2hiint(v), lo = (unsigned)__double2loint(v);
    const unsigned ah = hi & 0x7fffffffu;
    ok = ok && ah < 0x47f00000u;
    const unsigned f = (hi & 0x80000000u) | ((ah - 0x38000000u) << 3) | (lo >> 29);
    return ah < 0x38100000u ? 0.f : __uint_as_float(f);
}

// Where q = fl64(n / d) lies against [0, 1), given float32 values nf, df with
// |nf - n| <= E and |df - d| <= E: 1 inside, 0 outside, -1 undecided.
//  * d's sign is certain when |df| > E; with it, nn = nf sgn(d), dn = |df|
//    bound n sgn(d) in [nn - E, nn + E] and |d| in [dn - E, dn + E].
//  * q > 0 when nn - E > 0, and q < 0 when nn + E < 0 (then |q| is far above
//    the smallest double, so it does not round to -0).
//  * q < 1 - 2^-54, which rounds below 1, when (nn + E) / (dn - E) is at most
//    1 - 2^-16 (the two float roundings of the sums move that ratio by a
//    factor of at most (1 + 2^-24) / (1 - 2^-24)); q >= 1, which rounds to
//    at least 1, when nn - E >= (1 + 2^-16)(dn + E).
__device__ __forceinline__ int unit_quotient_filter(float nf, float df, float E) {
    const float dn = fabsf(df);
    if (!(dn > E)) return -1;
    const float nn = df < 0.f ? -nf : nf;
    const float lo = __fsub_rn(nn, E), hi = __fadd_rn(nn, E);
    if (hi < 0.f) return 0;
    if (lo >= __fmul_rn(1.0000152587890625f, __fadd_rn(dn, E))) return 0;
    if (lo > 0.f && hi <= __fmul_rn(0.9999847412109375f, __fsub_rn(dn, E))) return 1;
    return -1;
}

// Float32 decision of the crossing test of the walk's inside step (both
// quotients of seg_hit's determinants in [0, 1)) for segment (x1, y1) ->
// (x1 - dx12, y1 - dy12) and edge (x3, y3) -> (x4, y4), all truncated images
// of the doubles the FP64 test uses, m at least their largest magnitude:
// 1 crossed, 0 not crossed, -1 undecided.
// Error bound: each float difference is within D = 2^-22 m (1 + 2^-21) +
// 2^-24 |diff| (1 + 2^-22) of the FP64 difference (two truncations of at
// most 2^-23 of a coordinate, the float rounding, the FP64 rounding); with
// S the largest float difference, each float determinant is within
// 4 D S + 2 D^2 + 2^-22 S^2 (plus terms of order 2^-53 S^2) of the FP64 one.
// The code takes D = 2^-21 m + 2^-23 S and E = 1.0625 (4 D S + 2 D^2 +
// 2^-19 S^2): twice to eight times those terms, and 6 % for the float
// rounding of E itself.  S is kept in [2^-40, 2^40] (no float underflow or
// overflow in the products); otherwise undecided.
__device__ __forceinline__ int crossing_filter(float x1, float y1, float dx12, float dy12, float x3, float y3,
                                               float x4, float y4, float m) {
    const float x13 = __fsub_rn(x1, x3), y13 = __fsub_rn(y1, y3);
    const float x34 = __fsub_rn(x3, x4), y34 = __fsub_rn(y3, y4);
    const float S = fmaxf(fmaxf(fmaxf(fabsf(x13), fabsf(y13)), fmaxf(fabsf(x34), fabsf(y34))),
                          fmaxf(fabsf(dx12), fabsf(dy12)));
    if (!(S >= 9.094947e-13f && S <= 1.0995116e12f && m <= 1.0995116e12f)) return -1;  // 2^-40, 2^40
    const float T = __fsub_rn(__fmul_rn(x13, y34), __fmul_rn(y13, x34));
    const float U = __fsub_rn(__fmul_rn(dx12, y13), __fmul_rn(dy12, x13));
    const float D = __fsub_rn(__fmul_rn(dx12, y34), __fmul_rn(dy12, x34));
    const float dd = __fadd_rn(__fmul_rn(4.76837158e-7f, m), __fmul_rn(1.1920929e-7f, S));  // 2^-21 m + 2^-23 S
    const float E = __fmul_rn(1.0625f, __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(4.f, dd), S), __fmul_rn(__fmul_rn(2.f, dd), dd)),
                                                 __fmul_rn(__fmul_rn(1.9073486e-6f, S), S)));  // 2^-19
    const int in_t = unit_quotient_filter(T, D, E);
    if (in_t == 0) return 0;
    const int in_u = unit_quotient_filter(-U, D, E);
    if (in_u == 0) return 0;
    return (in_t == 1 && in_u == 1) ? 1 : -1;
}

// contribution of one boundary edge to the extended winding number of
// point_is_inside_polygon (geometry.py:737-829)
__device__ __forceinline__ double winding_term(double x, double y, double vx0, double vy0,
                                               double vx1, double vy1) {
    double x0 = dsub(vx0, x), y0 = dsub(vy0, y);
    double x1 = dsub(vx1, x), y1 = dsub(vy1, y);
    if (dmul(y0, y1) < 0) {
        double r = dadd(x0, ddiv(dmul(y0, dsub(x1, x0)), dsub(y0, y1)));
        if (r > 0) return (y0 < 0) ? 1.0 : -1.0;
        return (y0 < 0) ? -1.0 : 1.0;
    } else if (y0 == 0) {
        if (x0 > 0) {
            if (y1 > 0) return 0.5;
            if (y1 < 0) return -0.5;
        } else if (x0 < 0) {
            if (y1 < 0) return 0.5;
            if (y1 > 0) return -0.5;
        }
    } else if (y1 == 0) {
        if (x1 > 0) {
            if (y0 < 0) return 0.5;
            if (y0 > 0) return -0.5;
        } else if (x1 < 0) {
            if (y0 > 0) return 0.5;
            if (y0 < 0) return -0.5;
        }
    }
    return 0.0;
}

#ifdef RG_DEBUG
// Debug builds (-DRG_DEBUG, regridding_gb300._build.build(debug=True)): every
// grid read of the build is bounds-checked.  A read outside the array sets
// FLAG_BOUNDS here and yields NaN (no trap: the build runs to its end and
// the host turns the flag into RG_ERR_WALK).
__device__ unsigned g_debug_flags;
__device__ __forceinline__ bool debug_in_grid(int64_t i, int64_t j, int64_t nx, int64_t ny) {
    if (i >= 0 && j >= 0 && i < nx && j < ny) return true;
    atomicOr(&g_debug_flags, FLAG_BOUNDS);
    return false;
}
#define RG_GRID_READ(a, i, j) \
    (debug_in_grid(i, j, nx, ny) ? __ldg((a) + (i) * ny + (j)) : __longlong_as_double(0x7ff8000000000000ll))
#else
#define RG_GRID_READ(a, i, j) __ldg((a) + (i) * ny + (j))
#endif

struct Grid {
    const double* x;
    const double* y;
    int64_t nx, ny;
    __device__ __forceinline__ double X(int64_t i, int64_t j) const { return RG_GRID_READ(x, i, j); }
    __device__ __forceinline__ double Y(int64_t i, int64_t j) const { return RG_GRID_READ(y, i, j); }
};

// point_is_inside_polygon on the 4 vertices of cell (i, j) in the order
// (i,j), (i+1,j), (i+1,j+1), (i,j+1) (_grids.py:251-276)
__device__ bool cell_contains(const Grid& g, int64_t i, int64_t j, double px, double py) {
    double vx[4], vy[4];
    vx[0] = g.X(i, j);         vy[0] = g.Y(i, j);
    vx[1] = g.X(i + 1, j);     vy[1] = g.Y(i + 1, j);
    vx[2] = g.X(i + 1, j + 1); vy[2] = g.Y(i + 1, j + 1);
    vx[3] = g.X(i, j + 1);     vy[3] = g.Y(i, j + 1);
    double w = 0;
#pragma unroll
    for (int v = 0; v < 4; v++) {
        int p = (v + 3) & 3;
        w = w + winding_term(px, py, vx[p], vy[p], vx[v], vy[v]);
    }
    return w != 0;
}

// _index_of_point_local: _grids.py:282-349
__device__ void locate_local(const Grid& g, double px, double py, int64_t i0, int64_t j0,
                             int64_t* oi, int64_t* oj) {
    int64_t ncx = g.nx - 1, ncy = g.ny - 1;
    int64_t ia = i0 - 1 > 0 ? i0 - 1 : 0, ib = i0 + 2 < ncx ? i0 + 2 : ncx;
    int64_t ja = j0 - 1 > 0 ? j0 - 1 : 0, jb = j0 + 2 < ncy ? j0 + 2 : ncy;
    for (int64_t ii = ia; ii < ib; ii++)
        for (int64_t jj = ja; jj < jb; jj++)
            if (cell_contains(g, ii, jj, px, py)) {
                *oi = ii;
                *oj = jj;
                return;
            }
    *oi = MAXSIZE;
    *oj = MAXSIZE;
}

// _bilinear_interpolation: regridding/_interp_ndarray.py:226-269
__device__ double bilinear(const double* a, int64_t sx, int64_t sy, double x, double y) {
    int64_t x00 = (int64_t)floor(x), y00 = (int64_t)floor(y);
    if (x00 < 0) x00 = 0;
    else if (x00 > sx - 2) x00 = sx - 2;
    if (y00 < 0) y00 = 0;
    else if (y00 > sy - 2) y00 = sy - 2;
    double a00 = __ldg(a + x00 * sy + y00), a01 = __ldg(a + x00 * sy + y00 + 1);
    double a10 = __ldg(a + (x00 + 1) * sy + y00), a11 = __ldg(a + (x00 + 1) * sy + y00 + 1);
    double dx = dsub(x, (double)x00), dy = dsub(y, (double)y00);
    double w00 = dmul(dsub(1.0, dx), dsub(1.0, dy)), w01 = dmul(dsub(1.0, dx), dy);
    double w10 = dmul(dx, dsub(1.0, dy)), w11 = dmul(dx, dy);
    return dadd(dadd(dadd(dmul(a00, w00), dmul(a01, w01)), dmul(a10, w10)), dmul(a11, w11));
}

__device__ __forceinline__ bool floor_ok(double v) { return isfinite(v) && fabs(v) < 9.0e18; }

// index_of_point_secant: _grids.py:352-463.  Returns false when the upstream
// falls back to index_of_point_brute (singular Jacobian, no convergence, or an
// iterate the upstream could not floor).
__device__ bool locate_secant(const Grid& g, double px, double py, int64_t* oi, int64_t* oj) {
    const double h = 1e-3;
    int64_t sx = g.nx, sy = g.ny;
    double i = (double)sx / 2, j = (double)sy / 2;
    for (int it = 0; it < 100; it++) {
        double xv = bilinear(g.x, sx, sy, i, j);
        double yv = bilinear(g.y, sx, sy, i, j);
        if (!floor_ok(i) || !floor_ok(j)) return false;
        int64_t i0 = (int64_t)floor(i), j0 = (int64_t)floor(j);
        double ex = dsub(xv, px), ey = dsub(yv, py);
        if (i0 >= 0 && j0 >= 0 && i0 < sx - 1 && j0 < sy - 1) {
            if (cell_contains(g, i0, j0, px, py)) {
                locate_local(g, px, py, i0, j0, oi, oj);
                return true;
            }
        }
        if (fabs(ex) < 1e-10 && fabs(ey) < 1e-10) {
            locate_local(g, px, py, i0, j0, oi, oj);
            return true;
        }
        double dx_di = ddiv(dsub(bilinear(g.x, sx, sy, dadd(i, h), j), xv), h);
        double dx_dj = ddiv(dsub(bilinear(g.x, sx, sy, i, dadd(j, h)), xv), h);
        double dy_di = ddiv(dsub(bilinear(g.y, sx, sy, dadd(i, h), j), yv), h);
        double dy_dj = ddiv(dsub(bilinear(g.y, sx, sy, i, dadd(j, h)), yv), h);
        double det = dsub(dmul(dx_di, dy_dj), dmul(dx_dj, dy_di));
        if (det == 0) return false;
        double di = ddiv(dsub(dmul(dy_dj, ex), dmul(dx_dj, ey)), det);
        double dj = ddiv(dadd(dmul(-dy_di, ex), dmul(dx_di, ey)), det);
        i = dsub(i, di);
        j = dsub(j, dj);
    }
    return false;
}

// index_of_point_brute (_grids.py:218-279) by one warp: lanes test 32
// consecutive cells of the upstream (i outer, j inner) order per round and
// the first containing cell of the first round with a hit wins.
__device__ void locate_brute_warp(const Grid& g, double px, double py, int64_t* oi, int64_t* oj) {
    int lane = threadIdx.x & 31;
    int64_t ncx = g.nx - 1, ncy = g.ny - 1, ncells = ncx * ncy;
    for (int64_t base = 0; base < ncells; base += 32) {
        int64_t k = base + lane;
        bool hit = k < ncells && cell_contains(g, k / ncy, k % ncy, px, py);
        unsigned m = __ballot_sync(0xffffffffu, hit);
        if (m) {
            int64_t kk = base + __ffs(m) - 1;
            *oi = kk / ncy;
            *oj = kk % ncy;
            return;
        }
    }
    *oi = MAXSIZE;
    *oj = MAXSIZE;
}

// ---------------------------------------------------------------------------
// per-grid preparation
// ---------------------------------------------------------------------------

// grid_volume: _grids.py:50-140.  One thread per cell; the four contour terms
// are added in the upstream order (((0 - A) + B) - C) + D.
__device__ __forceinline__ double cell_area_at(const double* __restrict__ x, const double* __restrict__ y,
                                               int64_t ny, int64_t p, int64_t q) {
    double x00 = x[p * ny + q], y00 = y[p * ny + q];
    double x10 = x[(p + 1) * ny + q], y10 = y[(p + 1) * ny + q];
    double x01 = x[p * ny + q + 1], y01 = y[p * ny + q + 1];
    double x11 = x[(p + 1) * ny + q + 1], y11 = y[(p + 1) * ny + q + 1];
    // axis 0 (transposed, coordinates swapped)
    double A = dmul(dsub(dmul(y00, x10), dmul(y10, x00)), 0.5);
    double B = dmul(dsub(dmul(y01, x11), dmul(y11, x01)), 0.5);
    // axis 1
    double C = dmul(dsub(dmul(x00, y01), dmul(x01, y00)), 0.5);
    double D = dmul(dsub(dmul(x10, y11), dmul(x11, y10)), 0.5);
    double v = dsub(0.0, A);
    v = dadd(v, B);
    v = dsub(v, C);
    v = dadd(v, D);
    return v;
}

__global__ void cell_area_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                 int64_t nx, int64_t ny, double* __restrict__ out) {
    int64_t ncx = nx - 1, ncy = ny - 1;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncx * ncy;
         c += (int64_t)gridDim.x * blockDim.x)
        out[c] = cell_area_at(x, y, ny, c / ncy, c % ncy);
}

// Boundary edges in the scan order of _step_outside_static (:608-683):
// axis 0 (faces i = 0 then i = nx-1, running along j), then axis 1 (faces
// j = 0 then j = ny-1, running along i).
struct Edge {
    double x3, y3, x4, y4;
    int64_t cell;  // flat static cell index
    int code;      // direction_face * 2 + axis = the cell edge it enters through
    int pad;
};

__device__ __forceinline__ Edge boundary_edge(const Grid& g, int64_t k) {
    const int64_t ncx = g.nx - 1, ncy = g.ny - 1;
    int axis, dir;
    int64_t i0, kk = k;
    if (kk < 2 * ncy) {
        axis = 0;
        dir = kk >= ncy;
        i0 = kk - dir * ncy;
    } else {
        kk -= 2 * ncy;
        axis = 1;
        dir = kk >= ncx;
        i0 = kk - dir * ncx;
    }
    Edge e;
    if (axis == 0) {
        int64_t ie = dir ? g.nx - 1 : 0;
        e.x3 = g.X(ie, i0); e.y3 = g.Y(ie, i0);
        e.x4 = g.X(ie, i0 + 1); e.y4 = g.Y(ie, i0 + 1);
        int64_t cx = dir ? ncx - 1 : 0;
        e.cell = cx * ncy + i0;
    } else {
        int64_t je = dir ? g.ny - 1 : 0;
        e.x3 = g.X(i0, je); e.y3 = g.Y(i0, je);
        e.x4 = g.X(i0 + 1, je); e.y4 = g.Y(i0 + 1, je);
        int64_t cy = dir ? ncy - 1 : 0;
        e.cell = i0 * ncy + cy;
    }
    e.code = dir * 2 + axis;
    e.pad = 0;
    return e;
}

struct Bins {
    double ox, oy, inv_h;
    int nbx, nby;
    const int32_t* ptr;    // [nbx*nby + 1] offsets into items
    const int32_t* items;  // edge indices
};

__device__ __forceinline__ int bin_coord(double v, double o, double inv_h, int nb) {
    double f = floor(dmul(dsub(v, o), inv_h));
    if (!(f >= 0)) return 0;  // also maps NaN to 0
    if (f >= nb - 1) return nb - 1;
    return (int)f;
}

// Static-grid preparation of a whole batch.  The static grids are the input
// and the output grid of every pair (grid 2g and 2g + 1 for pair g); they
// share batch-wide arrays, so that every stage below is one launch whatever
// the number of pairs.  Grid k's boundary edges start at edge_base; its
// nbins + 1 bin slots (the last one always empty, so that the grid's slots
// end on its own total) start at bin_base.  Its bins hold offsets into the
// batch's one item array, and its items are edge indices of the grid.
struct PrepGrid {
    Grid g;
    Bins b;
    int64_t cell_base;  // first cell of the pair's input grid in area_in (even k only)
    int64_t edge_base;
    int64_t bin_base;
};

// grid k whose edges hold batch edge e (edge bases rise strictly: a grid has
// at least four boundary edges)
__device__ __forceinline__ int grid_of_edge(const PrepGrid* __restrict__ P, int n, int64_t e) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P[mid].edge_base <= e) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// areas of the input cells of every pair, in area_in's order (pair by pair)
__global__ void cell_area_batch(const PrepGrid* __restrict__ P, int G, int64_t ncells, double* __restrict__ out) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells;
         c += (int64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = G - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (P[2 * mid].cell_base <= c) lo = mid;
            else hi = mid - 1;
        }
        const Grid g = P[2 * lo].g;
        const int64_t local = c - P[2 * lo].cell_base, ncy = g.ny - 1;
        out[c] = cell_area_at(g.x, g.y, g.ny, local / ncy, local % ncy);
    }
}

// Bounding boxes (xmin, ymin, xmax, ymax) of every static grid: nparts
// blocks of 256 threads per grid fold strided vertices into partial
// extrema, then one warp per grid combines them (min and max are exact in
// any order, so the partition does not matter).
__global__ void __launch_bounds__(256) bbox_partial_batch(const PrepGrid* __restrict__ P, int nparts,
                                                          double* __restrict__ part) {
    __shared__ double sh[4][256];
    const int k = blockIdx.x / nparts, p = blockIdx.x % nparts;
    const Grid g = P[k].g;
    const int64_t n = g.nx * g.ny;
    double a = INFINITY, b = INFINITY, c = -INFINITY, d = -INFINITY;
    for (int64_t v = (int64_t)p * blockDim.x + threadIdx.x; v < n; v += (int64_t)nparts * blockDim.x) {
        const double xv = g.x[v], yv = g.y[v];
        a = fmin(a, xv);
        b = fmin(b, yv);
        c = fmax(c, xv);
        d = fmax(d, yv);
    }
    sh[0][threadIdx.x] = a;
    sh[1][threadIdx.x] = b;
    sh[2][threadIdx.x] = c;
    sh[3][threadIdx.x] = d;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            sh[0][threadIdx.x] = fmin(sh[0][threadIdx.x], sh[0][threadIdx.x + w]);
            sh[1][threadIdx.x] = fmin(sh[1][threadIdx.x], sh[1][threadIdx.x + w]);
            sh[2][threadIdx.x] = fmax(sh[2][threadIdx.x], sh[2][threadIdx.x + w]);
            sh[3][threadIdx.x] = fmax(sh[3][threadIdx.x], sh[3][threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x < 4) part[((int64_t)k * nparts + p) * 4 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void bbox_combine_batch(const double* __restrict__ part, int nparts, int ngrids, double* __restrict__ out) {
    const int k = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (k >= ngrids) return;  // whole warps leave together
    const double* q = part + (int64_t)k * nparts * 4;
    double a = INFINITY, b = INFINITY, c = -INFINITY, d = -INFINITY;
    for (int i = lane; i < nparts; i += 32) {
        a = fmin(a, q[4 * i]);
        b = fmin(b, q[4 * i + 1]);
        c = fmax(c, q[4 * i + 2]);
        d = fmax(d, q[4 * i + 3]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a = fmin(a, __shfl_xor_sync(0xffffffffu, a, o));
        b = fmin(b, __shfl_xor_sync(0xffffffffu, b, o));
        c = fmax(c, __shfl_xor_sync(0xffffffffu, c, o));
        d = fmax(d, __shfl_xor_sync(0xffffffffu, d, o));
    }
    if (lane == 0) {
        out[4 * k] = a;
        out[4 * k + 1] = b;
        out[4 * k + 2] = c;
        out[4 * k + 3] = d;
    }
}

__global__ void boundary_edges_batch(const PrepGrid* __restrict__ P, int ngrids, int64_t nedges,
                                     Edge* __restrict__ edges) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nedges;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int k = grid_of_edge(P, ngrids, e);
        edges[e] = boundary_edge(P[k].g, e - P[k].edge_base);
    }
}

// Every edge goes to each bin its bounding box touches: a counting pass,
// then (after the scan of the counts) a filing pass.  The order of the
// items within a bin depends on the atomics; the outside step that reads
// them is order-independent.
template <bool FILL>
__global__ void bin_edges_batch(const PrepGrid* __restrict__ P, int ngrids, const Edge* __restrict__ edges,
                                int64_t nedges, unsigned* __restrict__ counts, int32_t* __restrict__ items,
                                const int64_t* __restrict__ ptr64) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nedges;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int gk = grid_of_edge(P, ngrids, k);
        const Bins b = P[gk].b;
        const int64_t base = P[gk].bin_base;
        const Edge e = edges[k];
        int bx0 = bin_coord(fmin(e.x3, e.x4), b.ox, b.inv_h, b.nbx);
        int bx1 = bin_coord(fmax(e.x3, e.x4), b.ox, b.inv_h, b.nbx);
        int by0 = bin_coord(fmin(e.y3, e.y4), b.oy, b.inv_h, b.nby);
        int by1 = bin_coord(fmax(e.y3, e.y4), b.oy, b.inv_h, b.nby);
        for (int by = by0; by <= by1; by++)
            for (int bx = bx0; bx <= bx1; bx++) {
                const int64_t bin = base + (int64_t)by * b.nbx + bx;
                unsigned pos = atomicAdd(&counts[bin], 1u);
                if (FILL) items[ptr64[bin] + pos] = (int32_t)(k - P[gk].edge_base);
            }
    }
}

__global__ void i64_to_i32(const int64_t* a, int32_t* b, int64_t n) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        b[k] = (int32_t)a[k];
}

// ---------------------------------------------------------------------------
// sweep families and line seats
// ---------------------------------------------------------------------------

struct Static {
    Grid g;
    int64_t ncx, ncy;
    double blx, bly, bux, buy;
    int64_t nbound;  // boundary polygon vertices
    const Edge* edges;
    Bins bins;
};

struct Family {
    Grid sweep;        // unaligned sweep grid
    int transposed;    // axis_sweep == 0
    int64_t lines;     // aligned rows
    int64_t len;       // aligned columns (vertices along a line)
    int sweep_input;
    int axis;
    int st;            // 0: static = input grid, 1: static = output grid
    int64_t line_base;
    __device__ __forceinline__ double SX(int64_t a, int64_t b) const {
        return transposed ? sweep.X(b, a) : sweep.X(a, b);
    }
    __device__ __forceinline__ double SY(int64_t a, int64_t b) const {
        return transposed ? sweep.Y(b, a) : sweep.Y(a, b);
    }
};

struct SweepParams {
    Family fam[4];
    Static st[2];
    const double* area_in;  // (ncx_in, ncy_in)
    const double* w_in;     // nullable
    int64_t ncy_in, ncy_out;
    int64_t total_lines;
};

struct Seat {
    int64_t stx, sty;
    int outside;
    int pad;
};

__device__ __forceinline__ int family_of(const SweepParams& P, int64_t line) {
    int f = 0;
#pragma unroll
    for (int k = 1; k < 4; k++)
        if (line >= P.fam[k].line_base) f = k;
    return f;
}

// A batch of grid pairs swept together: per pair its sweep parameters and
// chunk plan (whose line, chunk and slot bases are global across the batch),
// prefix bases of its lines, chunks and output rows, and its own error word.
// Kernels find their pair by binary search over the prefix bases.
struct ChunkPlan;
struct Batch {
    const SweepParams* P;    // [G]
    const ChunkPlan* C;      // [G] (null for whole-line walks)
    const int64_t* line_base;   // [G + 1]
    const int64_t* chunk_base;  // [G + 1]
    const int64_t* out_base;    // [G + 1] first output row of every pair
    unsigned* flags;            // [G]
    int G;
};

// the pair owning global index x: the largest g with base[g] <= x
__device__ __forceinline__ int pair_of(const int64_t* __restrict__ base, int G, int64_t x) {
    int lo = 0, hi = G - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (base[mid] <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Starting state of every sweep line (:439-468): one warp per line.
__global__ void __launch_bounds__(128) seat_kernel(Batch B, Seat* seats) {
    int lane = threadIdx.x & 31;
    int64_t line = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (line >= B.line_base[B.G]) return;
    const int pg = pair_of(B.line_base, B.G, line);
    const SweepParams& P = B.P[pg];
    unsigned* flags = B.flags + pg;
    const Family& F = P.fam[family_of(P, line)];
    const Static& S = P.st[F.st];
    int64_t li = line - F.line_base;
    double x1 = F.SX(li, 0), y1 = F.SY(li, 0);
    Seat seat;
    seat.stx = MAXSIZE;
    seat.sty = MAXSIZE;
    seat.outside = 1;
    seat.pad = 0;
    bool in_box = (S.blx <= x1 && x1 <= S.bux) && (S.bly <= y1 && y1 <= S.buy);
    if (in_box) {
        // Winding number of the boundary polygon at the line's first vertex.
        // Only edges whose y-range holds y1 have a nonzero term, and all of
        // them lie in the row of edge bins at y1's bin (bin_coord is
        // monotone); an edge spanning several x-bins of the row is counted
        // in its first.  The boundary edges run along the polygon's order on
        // the faces j = 0 and i = nx - 1 and against it on i = 0 and
        // j = ny - 1 (codes 0 and 3), where their ends are swapped back.
        // The terms are 0, +-1/2 and +-1, so the sum is exact in any order.
        double w = 0;
        const Bins& BN = S.bins;
        const int row = bin_coord(y1, BN.oy, BN.inv_h, BN.nby);
        for (int bx = lane; bx < BN.nbx; bx += 32) {
            const int64_t bin = (int64_t)row * BN.nbx + bx;
            const int32_t q0 = __ldg(BN.ptr + bin), q1 = __ldg(BN.ptr + bin + 1);
            for (int32_t q = q0; q < q1; q++) {
                const Edge e = S.edges[__ldg(BN.items + q)];
                if (bin_coord(fmin(e.x3, e.x4), BN.ox, BN.inv_h, BN.nbx) != bx) continue;
                if (e.code == 0 || e.code == 3) w += winding_term(x1, y1, e.x4, e.y4, e.x3, e.y3);
                else w += winding_term(x1, y1, e.x3, e.y3, e.x4, e.y4);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
        if (w != 0) {
            int64_t i = MAXSIZE, j = MAXSIZE;
            int ok = 0;
            if (lane == 0) ok = locate_secant(S.g, x1, y1, &i, &j);
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) locate_brute_warp(S.g, x1, y1, &i, &j);
            if (i == MAXSIZE) {
                // the upstream would index out of range here; report it and
                // leave the line outside so the walk stays in bounds
                if (lane == 0) atomicOr(flags, FLAG_SEAT_OUTSIDE);
            } else {
                seat.stx = i;
                seat.sty = j;
                seat.outside = 0;
            }
        }
    }
    if (lane == 0) seats[line] = seat;
}

// ---------------------------------------------------------------------------
// the walk
// ---------------------------------------------------------------------------

__constant__ int c_vtx_i[4] = {0, 1, 1, 0};   // indices_cell_vertex: _grids.py:153-158
__constant__ int c_vtx_j[4] = {0, 0, 1, 1};
__constant__ int c_nrm_i[4] = {-1, 0, 1, 0};  // cell_normals: _grids.py:143-148
__constant__ int c_nrm_j[4] = {0, -1, 0, 1};

// State of a walk at a sweep vertex.  At every vertex the upstream's
// entry-edge marker is back at sys.maxsize and the current point is the
// vertex itself, so (outside, static cell) is the whole state.
struct WalkState {
    int64_t stx, sty;
    int64_t sy;  // index of the sweep vertex the walk is at
    int outside;
    int pad;
};

// The body of the prange loop of _sweep_along_axis (:432-533) with
// _step_outside_static (:547-698), _step_inside_static (:707-895) and
// _calc_and_save_weights (:903-976) inlined, run on line li from vertex
// st.sy until the walk reaches vertex j_end.  WRITE stores triples at
// [wpos, wend); past wend it only counts (and flags the overflow).  Returns
// the number of triples emitted.
template <bool WRITE>
__device__ int64_t walk_range(const SweepParams& P, const Family& F, const Static& S, int64_t li, int64_t j_end,
                              WalkState& state, int64_t wpos, int64_t wend, int32_t* __restrict__ raw_in,
                              int32_t* __restrict__ raw_out, double* __restrict__ raw_val, unsigned* flags,
                              int64_t max_steps) {
    const Grid st = S.g;
    int64_t stx = state.stx, sty = state.sty;
    bool outside = state.outside;
    int64_t edge_last = MAXSIZE;
    int64_t sy_idx = state.sy;
    int64_t n_emit = 0;
    int64_t steps = 0;
    double x1 = F.SX(li, sy_idx), y1 = F.SY(li, sy_idx);

    while (sy_idx < j_end) {
        if (++steps > max_steps) {
            atomicOr(flags, FLAG_WALK_CAP);
            break;
        }
        double x2 = F.SX(li, sy_idx + 1), y2 = F.SY(li, sy_idx + 1);
        if (outside) {
            // _step_outside_static: smallest-t crossing of the static boundary,
            // candidates from the bins overlapping the segment's box
            const double p2x = x2, p2y = y2;
            double sminx = fmin(x1, p2x), smaxx = fmax(x1, p2x);
            double sminy = fmin(y1, p2y), smaxy = fmax(y1, p2y);
            bool found = false;
            double t_min = INFINITY;
            // float32 images of the segment for the crossing filter
            bool seg_ok = true;
            const float x1f = trunc_float(x1, seg_ok), y1f = trunc_float(y1, seg_ok);
            const float x2f = trunc_float(p2x, seg_ok), y2f = trunc_float(p2y, seg_ok);
            const float dx12f = __fsub_rn(x1f, x2f), dy12f = __fsub_rn(y1f, y2f);
            const float mseg = fmaxf(fmaxf(fabsf(x1f), fabsf(y1f)), fmaxf(fabsf(x2f), fabsf(y2f)));
            int64_t best_order = INT64_MAX;
            int best_code = 0;
            int64_t best_cell = 0;
            if (!(smaxx < S.blx || sminx > S.bux || smaxy < S.bly || sminy > S.buy)) {
                const Bins& B = S.bins;
                int bx0 = bin_coord(sminx, B.ox, B.inv_h, B.nbx);
                int bx1 = bin_coord(smaxx, B.ox, B.inv_h, B.nbx);
                int by0 = bin_coord(sminy, B.oy, B.inv_h, B.nby);
                int by1 = bin_coord(smaxy, B.oy, B.inv_h, B.nby);
                for (int by = by0; by <= by1; by++) {
                    for (int bx = bx0; bx <= bx1; bx++) {
                        int64_t bin = (int64_t)by * B.nbx + bx;
                        int32_t s0 = __ldg(B.ptr + bin), s1 = __ldg(B.ptr + bin + 1);
                        for (int32_t q = s0; q < s1; q++) {
                            int32_t ek = __ldg(B.items + q);
                            const Edge e = S.edges[ek];
                            if (!bboxes_intersect(x1, y1, p2x, p2y, e.x3, e.y3, e.x4, e.y4)) continue;
                            {
                                // most candidate boundary edges are certainly not crossed
                                bool ok = seg_ok;
                                const float x3f = trunc_float(e.x3, ok), y3f = trunc_float(e.y3, ok);
                                const float x4f = trunc_float(e.x4, ok), y4f = trunc_float(e.y4, ok);
                                const float m = fmaxf(mseg, fmaxf(fmaxf(fabsf(x3f), fabsf(y3f)),
                                                                  fmaxf(fabsf(x4f), fabsf(y4f))));
                                if (ok && crossing_filter(x1f, y1f, dx12f, dy12f, x3f, y3f, x4f, y4f, m) == 0) continue;
                            }
                            double t;
                            if (!seg_hit(x1, y1, p2x, p2y, e.x3, e.y3, e.x4, e.y4, &t)) continue;
                            if (e.cell == edge_last) continue;
                            if (t < t_min || (t == t_min && ek < best_order)) {
                                t_min = t;
                                best_order = ek;
                                best_code = e.code;
                                best_cell = e.cell;
                                found = true;
                            }
                        }
                    }
                }
            }
            if (found) {
                stx = best_cell / S.ncy;
                sty = best_cell % S.ncy;
                x2 = dadd(x1, dmul(t_min, dsub(p2x, x1)));
                y2 = dadd(y1, dmul(t_min, dsub(p2y, y1)));
                edge_last = best_code;
                outside = false;
            } else {
                edge_last = MAXSIZE;
                sy_idx = sy_idx + 1;
            }
        } else {
            // _step_inside_static: first crossed edge of the current static
            // cell other than the entry edge
            // The hit test of each candidate edge is seg_hit's, with the two
            // quotients placed against [0, 1) on their bits where that is
            // certain (almost always); only the edge found needs its crossing
            // parameter divided out.  Same edges, same order, same t.
            const double p2x = x2, p2y = y2;
            const double dx12 = dsub(x1, p2x), dy12 = dsub(y1, p2y);
            int found = -1;
            double f_tdet = 0.0, f_det = 1.0;
            // float32 images of the segment for the crossing filter
            bool seg_ok = true;
            const float x1f = trunc_float(x1, seg_ok), y1f = trunc_float(y1, seg_ok);
            const float x2f = trunc_float(p2x, seg_ok), y2f = trunc_float(p2y, seg_ok);
            const float dx12f = __fsub_rn(x1f, x2f), dy12f = __fsub_rn(y1f, y2f);
            const float mseg = fmaxf(fmaxf(fabsf(x1f), fabsf(y1f)), fmaxf(fabsf(x2f), fabsf(y2f)));
#pragma unroll 1
            for (int v = 0; v < 4; v++) {
                if (v == edge_last) continue;
                int vp = (v + 3) & 3;
                double x3 = st.X(stx + c_vtx_i[vp], sty + c_vtx_j[vp]);
                double y3 = st.Y(stx + c_vtx_i[vp], sty + c_vtx_j[vp]);
                double x4 = st.X(stx + c_vtx_i[v], sty + c_vtx_j[v]);
                double y4 = st.Y(stx + c_vtx_i[v], sty + c_vtx_j[v]);
                if (!bboxes_intersect(x1, y1, p2x, p2y, x3, y3, x4, y4)) continue;
                // 1: crossed, 0: not crossed (both certain), -1: the FP64 test decides
                int dec = -1;
                {
                    bool ok = seg_ok;
                    const float x3f = trunc_float(x3, ok), y3f = trunc_float(y3, ok);
                    const float x4f = trunc_float(x4, ok), y4f = trunc_float(y4, ok);
                    const float m = fmaxf(mseg, fmaxf(fmaxf(fabsf(x3f), fabsf(y3f)), fmaxf(fabsf(x4f), fabsf(y4f))));
                    if (ok) dec = crossing_filter(x1f, y1f, dx12f, dy12f, x3f, y3f, x4f, y4f, m);
                }
                if (dec == 0) continue;
                const double x13 = dsub(x1, x3), y13 = dsub(y1, y3);
                const double x34 = dsub(x3, x4), y34 = dsub(y3, y4);
                const double tdet = dsub(dmul(x13, y34), dmul(y13, x34));
                const double det = dsub(dmul(dx12, y34), dmul(dy12, x34));
                if (dec < 0) {
                    const double udet = dsub(dmul(dx12, y13), dmul(dy12, x13));
                    const int in_t = quotient_in_unit(tdet, det);
                    const int in_u = quotient_in_unit(-udet, det);
                    if (in_t == 0 || in_u == 0) continue;
                    if (in_t < 0 || in_u < 0) {
                        const double t = ddiv(tdet, det), u = ddiv(-udet, det);
                        if (!((0 <= t && t < 1) && (0 <= u && u < 1))) continue;
                    }
                }
                found = v;
                f_tdet = tdet;
                f_det = det;
                break;
            }
            if (found >= 0) {
                const double t = ddiv(f_tdet, f_det);
                x2 = dadd(x1, dmul(t, dsub(p2x, x1)));
                y2 = dadd(y1, dmul(t, dsub(p2y, y1)));
            }
            int64_t nsy, nstx, nsty;
            if (found >= 0) {
                nsy = sy_idx;
                nstx = stx + c_nrm_i[found];
                nsty = sty + c_nrm_j[found];
                edge_last = (found + 2) % 4;
            } else {
                nsy = sy_idx + 1;
                nstx = stx;
                nsty = sty;
                edge_last = MAXSIZE;
            }
            // _calc_and_save_weights: area_triangle, negated for axis 0
            double area = dmul(dsub(dmul(x1, y2), dmul(x2, y1)), 0.5);
            if (F.axis == 0) area = -area;
            // when the static grid is the input grid both sides share the
            // input cell, and -area / a_in (times w_in) is exactly the
            // negation of area / a_in (times w_in): one division serves both
            double w_static = 0.0;
            bool have_static = false;
#pragma unroll
            for (int side = 0; side < 2; side++) {
                int64_t is = side == 0 ? li - 1 : li;
                if (side == 0 && !(is >= 0)) continue;
                if (side == 1 && !(is < F.lines - 1)) continue;
                int64_t a = is, b = sy_idx;
                if (F.axis == 0) { a = sy_idx; b = is; }
                int64_t ii, ij, oi, oj;
                if (F.sweep_input) { ii = a; ij = b; oi = stx; oj = sty; }
                else { ii = stx; ij = sty; oi = a; oj = b; }
                int64_t in_flat = ii * P.ncy_in + ij;
                if (WRITE) {
                    if (wpos < wend) {
                        double w;
                        if (!F.sweep_input && have_static) {
                            w = -w_static;
                        } else {
                            double ain = __ldg(P.area_in + in_flat);
                            w = side == 0 ? ddiv(area, ain) : ddiv(-area, ain);
                            if (P.w_in) w = dmul(w, __ldg(P.w_in + in_flat));
                            if (!F.sweep_input && side == 0) {
                                w_static = w;
                                have_static = true;
                            }
                        }
                        raw_in[wpos] = (int32_t)in_flat;
                        raw_out[wpos] = (int32_t)(oi * P.ncy_out + oj);
                        raw_val[wpos] = w;
                    } else {
                        // never write past the slots given to this walk
                        atomicOr(flags, FLAG_CAPACITY);
                    }
                    wpos++;
                }
                n_emit++;
            }
            if (!(nstx >= 0 && nsty >= 0 && nstx < S.ncx && nsty < S.ncy)) {
                edge_last = stx * S.ncy + sty;
                nstx = MAXSIZE;
                nsty = MAXSIZE;
                outside = true;
            }
            sy_idx = nsy;
            stx = nstx;
            sty = nsty;
        }
        x1 = x2;
        y1 = y2;
    }
    state.stx = stx;
    state.sty = sty;
    state.sy = sy_idx;
    state.outside = outside;
    return n_emit;
}

// One thread per sweep line over the whole line.  COUNT mode only counts the
// triples a line emits; WRITE mode stores them from offsets[line].
template <bool WRITE>
__global__ void __launch_bounds__(64)
    walk_kernel(Batch B, const Seat* __restrict__ seats, int64_t* __restrict__ counts,
                const int64_t* __restrict__ offsets, int32_t* __restrict__ raw_in,
                int32_t* __restrict__ raw_out, double* __restrict__ raw_val) {
    int64_t line = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (line >= B.line_base[B.G]) return;
    const int pg = pair_of(B.line_base, B.G, line);
    const SweepParams& P = B.P[pg];
    const Family F = P.fam[family_of(P, line)];
    const Static& S = P.st[F.st];
    Seat seat = seats[line];
    WalkState state{seat.stx, seat.sty, 0, seat.outside, 0};
    const int64_t max_steps = 64 * (F.len + 4 * (S.ncx + S.ncy) + 16);
    int64_t n = walk_range<WRITE>(P, F, S, line - F.line_base, F.len - 1, state,
                                  WRITE ? offsets[line] : 0, WRITE ? offsets[line + 1] : 0, raw_in, raw_out,
                                  raw_val, B.flags + pg, max_steps);
    if (!WRITE) counts[line] = n;
    if (WRITE && B.out_base[pg] != 0) {
        // output rows of the batch: the pair's rows follow those of the pairs before it
        const int32_t ob = (int32_t)B.out_base[pg];
        for (int64_t q = offsets[line]; q < offsets[line] + n; q++) raw_out[q] += ob;
    }
}

// ---------------------------------------------------------------------------
// chunked walk: every line is cut into chunks of CH sweep segments that are
// walked in parallel.  A chunk starts from its vertex located in the static
// grid; a per-line repair pass then re-walks, in order, every chunk whose
// start disagrees with the end state of the chunk before it, so the triples
// are exactly those of one sequential walk per line.
// ---------------------------------------------------------------------------

struct ChunkPlan {
    int64_t ch;              // sweep segments per chunk
    int64_t nc[4];           // chunks per line, per family
    int64_t chunk_base[5];   // first chunk id of each family (and the total)
    int64_t cap[4];          // triple slots per chunk, per family
    int64_t slot_base[4];    // first slot of each family
};

__device__ __forceinline__ int family_of_chunk(const ChunkPlan& C, int64_t g) {
    int f = 0;
#pragma unroll
    for (int k = 1; k < 4; k++)
        if (g >= C.chunk_base[k]) f = k;
    return f;
}

// A guess of the walk state at a sweep vertex: the static cell containing
// it (Newton seed on the bilinear index map, then a walk across the edge the
// point lies beyond), or "outside".  Wrong guesses are fixed by the repair.
__device__ WalkState guess_state(const Static& S, double px, double py, int64_t sy) {
    WalkState w{MAXSIZE, MAXSIZE, sy, 1, 0};
    if (!((S.blx <= px && px <= S.bux) && (S.bly <= py && py <= S.buy))) return w;
    const Grid& g = S.g;
    const int64_t ncx = S.ncx, ncy = S.ncy;
    int64_t ci, cj;
    seed_cell(g.x, g.y, g.nx, g.ny, px, py, &ci, &cj);
    for (int step = 0; step < 64; step++) {
        if (cell_contains(g, ci, cj, px, py)) {
            w.stx = ci;
            w.sty = cj;
            w.outside = 0;
            return w;
        }
        double vx[4] = {g.X(ci, cj), g.X(ci + 1, cj), g.X(ci + 1, cj + 1), g.X(ci, cj + 1)};
        double vy[4] = {g.Y(ci, cj), g.Y(ci + 1, cj), g.Y(ci + 1, cj + 1), g.Y(ci, cj + 1)};
        double area2 = (vx[0] - vx[2]) * (vy[1] - vy[3]) - (vx[1] - vx[3]) * (vy[0] - vy[2]);
        double sgn = area2 >= 0 ? 1.0 : -1.0;
        int best = -1;
        double worst = 0;
#pragma unroll
        for (int e = 0; e < 4; e++) {
            int f = (e + 1) & 3;
            double ex = vx[f] - vx[e], ey = vy[f] - vy[e];
            double cr = sgn * (ex * (py - vy[e]) - ey * (px - vx[e]));
            double len = sqrt(ex * ex + ey * ey);
            double sc = len > 0 ? cr / len : 0;
            if (sc < worst) {
                worst = sc;
                best = e;
            }
        }
        if (best < 0) break;
        const int di[4] = {0, 1, 0, -1};
        const int dj[4] = {-1, 0, 1, 0};
        int64_t ni = ci + di[best], nj = cj + dj[best];
        if (ni < 0 || nj < 0 || ni >= ncx || nj >= ncy) break;
        ci = ni;
        cj = nj;
    }
    return w;
}

__global__ void chunk_seat_kernel(Batch B, const Seat* __restrict__ seats, WalkState* __restrict__ starts) {
    int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= B.chunk_base[B.G]) return;
    const int pg = pair_of(B.chunk_base, B.G, g);
    const SweepParams& P = B.P[pg];
    const ChunkPlan& C = B.C[pg];
    int f = family_of_chunk(C, g);
    const Family& F = P.fam[f];
    int64_t k = g - C.chunk_base[f];
    int64_t li = k / C.nc[f], c = k - li * C.nc[f];
    int64_t j0 = c * C.ch;
    if (c == 0) {
        Seat s0 = seats[F.line_base + li];
        starts[g] = WalkState{s0.stx, s0.sty, 0, s0.outside, 0};
    } else {
        starts[g] = guess_state(P.st[F.st], F.SX(li, j0), F.SY(li, j0), j0);
    }
}

__device__ __forceinline__ int64_t chunk_end(const ChunkPlan& C, const Family& F, int64_t c) {
    int64_t e = (c + 1) * C.ch;
    return e < F.len - 1 ? e : F.len - 1;
}

__device__ __forceinline__ void chunk_walk_one(const Batch& B, const WalkState* __restrict__ starts,
                                               WalkState* __restrict__ ends, int64_t* __restrict__ counts,
                                               int32_t* __restrict__ s_in, int32_t* __restrict__ s_out,
                                               double* __restrict__ s_val, int64_t g) {
    const int pg = pair_of(B.chunk_base, B.G, g);
    const SweepParams& P = B.P[pg];
    const ChunkPlan& C = B.C[pg];
    unsigned* flags = B.flags + pg;
    int f = family_of_chunk(C, g);
    const Family F = P.fam[f];
    const Static& S = P.st[F.st];
    int64_t k = g - C.chunk_base[f];
    int64_t li = k / C.nc[f], c = k - li * C.nc[f];
    WalkState st = starts[g];
    int64_t base = C.slot_base[f] + k * C.cap[f];
    const int64_t max_steps = 64 * (C.ch + 4 * (S.ncx + S.ncy) + 16);
    counts[g] = walk_range<true>(P, F, S, li, chunk_end(C, F, c), st, base, base + C.cap[f], s_in, s_out,
                                 s_val, flags, max_steps);
    ends[g] = st;
}

// Chunks are handed out one at a time from a counter: a thread that finishes
// a short chunk takes the next one instead of idling until the longest chunk
// of its warp is done (walk lengths differ between chunks).
__global__ void __launch_bounds__(64)
    chunk_walk_kernel(Batch B, const WalkState* __restrict__ starts, WalkState* __restrict__ ends,
                      int64_t* __restrict__ counts, int32_t* __restrict__ s_in, int32_t* __restrict__ s_out,
                      double* __restrict__ s_val, unsigned long long* __restrict__ next_chunk) {
    const int64_t total = B.chunk_base[B.G];
    for (;;) {
        const int64_t g = (int64_t)atomicAdd(next_chunk, 1ull);
        if (g >= total) return;
        chunk_walk_one(B, starts, ends, counts, s_in, s_out, s_val, g);
    }
}

// One thread per line: walk chunks again, in order, wherever a chunk's start
// differs from the previous chunk's end.
__global__ void __launch_bounds__(64)
    chunk_repair_kernel(Batch B, WalkState* __restrict__ starts, WalkState* __restrict__ ends,
                        int64_t* __restrict__ counts, int32_t* __restrict__ s_in, int32_t* __restrict__ s_out,
                        double* __restrict__ s_val, unsigned long long* __restrict__ n_repaired) {
    int64_t line = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (line >= B.line_base[B.G]) return;
    const int pg = pair_of(B.line_base, B.G, line);
    const SweepParams& P = B.P[pg];
    const ChunkPlan& C = B.C[pg];
    unsigned* flags = B.flags + pg;
    int f = family_of(P, line);
    const Family F = P.fam[f];
    const Static& S = P.st[F.st];
    int64_t li = line - F.line_base;
    const int64_t max_steps = 64 * (C.ch + 4 * (S.ncx + S.ncy) + 16);
    int64_t g0 = C.chunk_base[f] + li * C.nc[f];
    for (int64_t c = 1; c < C.nc[f]; c++) {
        WalkState prev = ends[g0 + c - 1];
        WalkState cur = starts[g0 + c];
        bool same = prev.outside == cur.outside && (prev.outside || (prev.stx == cur.stx && prev.sty == cur.sty));
        if (same) continue;
        atomicAdd(n_repaired, 1ull);
        starts[g0 + c] = prev;
        WalkState st = prev;
        int64_t k = li * C.nc[f] + c;
        int64_t base = C.slot_base[f] + k * C.cap[f];
        counts[g0 + c] = walk_range<true>(P, F, S, li, chunk_end(C, F, c), st, base, base + C.cap[f], s_in,
                                          s_out, s_val, flags, max_steps);
        ends[g0 + c] = st;
    }
}

// One warp per chunk: move its triples from its slots to their place in the
// emission order.

// ---------------------------------------------------------------------------
// merge (regridding/_weights/_weights_arrays.py:44-73)
// ---------------------------------------------------------------------------

// ---------------------------------------------------------------------------
// Output-row ordering of the chunked walk's triples, read straight from the
// chunks' slots (no compacted copy, no index indirection): chunk g's q-th
// triple has raw position offsets[g] + q (the order of one sequential walk
// per line), and it goes to the bucket of its output row with the key
// (input cell << 32 | raw position), so that ordering each row by key gives
// the same order as the bucket sort of the compacted triples: by input
// cell, then by raw position.  One warp per chunk in the counting and
// scattering passes (a chunk's consecutive triples often share a row, and
// their lanes add to its counter once), one warp per row in the ranking.
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned warp_row_add(unsigned* counters, int32_t b, bool active) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned key = active ? (unsigned)b : 0xffffffffu;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const unsigned leader = __ffs(peers) - 1;
    unsigned base = 0;
    if (active && lane == leader) base = atomicAdd(&counters[b], (unsigned)__popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + __popc(peers & ((1u << lane) - 1u));
}

__global__ void slot_count_rows(Batch B, const int64_t* __restrict__ counts, const int32_t* __restrict__ s_out,
                                unsigned* __restrict__ rows) {
    const int lane = threadIdx.x & 31;
    const int64_t g = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (g >= B.chunk_base[B.G]) return;  // warp-uniform
    const int pg = pair_of(B.chunk_base, B.G, g);
    const ChunkPlan& C = B.C[pg];
    const int32_t ob = (int32_t)B.out_base[pg];
    const int f = family_of_chunk(C, g);
    const int64_t base = C.slot_base[f] + (g - C.chunk_base[f]) * C.cap[f];
    const int64_t n = counts[g];
    for (int64_t q0 = 0; q0 < n; q0 += 32) {
        const int64_t q = q0 + lane;
        const bool active = q < n;
        (void)warp_row_add(rows, active ? s_out[base + q] + ob : 0, active);
    }
}

__global__ void slot_scatter_rows(Batch B, const int64_t* __restrict__ counts, const int64_t* __restrict__ offsets,
                                  const int32_t* __restrict__ s_in, const int32_t* __restrict__ s_out,
                                  const double* __restrict__ s_val, const int64_t* __restrict__ row_start,
                                  unsigned* __restrict__ cursor, int64_t* __restrict__ tkey,
                                  double* __restrict__ tval) {
    const int lane = threadIdx.x & 31;
    const int64_t g = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (g >= B.chunk_base[B.G]) return;  // warp-uniform
    const int pg = pair_of(B.chunk_base, B.G, g);
    const ChunkPlan& C = B.C[pg];
    const int32_t ob = (int32_t)B.out_base[pg];
    const int f = family_of_chunk(C, g);
    const int64_t base = C.slot_base[f] + (g - C.chunk_base[f]) * C.cap[f];
    const int64_t n = counts[g], raw0 = offsets[g];
    for (int64_t q0 = 0; q0 < n; q0 += 32) {
        const int64_t q = q0 + lane;
        const bool active = q < n;
        const int32_t b = active ? s_out[base + q] + ob : 0;
        const unsigned pos = warp_row_add(cursor, b, active);
        if (active) {
            const int64_t dst = row_start[b] + pos;
            tkey[dst] = ((int64_t)s_in[base + q] << 32) | (int64_t)(uint32_t)(raw0 + q);
            tval[dst] = s_val[base + q];
        }
    }
}

constexpr int ROW_SMALL = 64;  // rows ranked by one warp (two keys per lane)

// One warp per output row of at most ROW_SMALL triples: each triple's rank
// is the number of keys of its row below its own (keys are unique); the row
// is written out in that order.  Longer rows are listed for rank_rows_long.
__global__ void rank_rows(const int64_t* __restrict__ row_start, int64_t nrows, const int64_t* __restrict__ tkey,
                          const double* __restrict__ tval, int32_t* __restrict__ out_in,
                          double* __restrict__ out_val, int32_t* __restrict__ long_list,
                          unsigned* __restrict__ long_count) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < nrows; r += nwarps) {
        const int64_t s = row_start[r], n = row_start[r + 1] - s;  // warp-uniform
        if (n > ROW_SMALL) {
            if (lane == 0) long_list[atomicAdd(long_count, 1u)] = (int32_t)r;
            continue;
        }
        const int64_t k0 = lane < n ? tkey[s + lane] : INT64_MAX;
        const int64_t k1 = lane + 32 < n ? tkey[s + 32 + lane] : INT64_MAX;
        int r0 = 0, r1 = 0;
        const int n0 = n < 32 ? (int)n : 32;
        for (int j = 0; j < n0; j++) {
            const int64_t kj = __shfl_sync(0xffffffffu, k0, j);
            r0 += kj < k0;
            r1 += kj < k1;
        }
        for (int j = 32; j < n; j++) {
            const int64_t kj = __shfl_sync(0xffffffffu, k1, j - 32);
            r0 += kj < k0;
            r1 += kj < k1;
        }
        if (lane < n) {
            out_in[s + r0] = (int32_t)(k0 >> 32);
            out_val[s + r0] = tval[s + lane];
        }
        if (lane + 32 < n) {
            out_in[s + r1] = (int32_t)(k1 >> 32);
            out_val[s + r1] = tval[s + 32 + lane];
        }
    }
}

// One block per listed long row: keys staged in shared-memory tiles, every
// thread ranks up to 8 triples per pass.
constexpr int ROW_TILE = 2048;
__global__ void __launch_bounds__(256)
    rank_rows_long(const int64_t* __restrict__ row_start, const int32_t* __restrict__ long_list,
                   const unsigned* __restrict__ long_count, const int64_t* __restrict__ tkey,
                   const double* __restrict__ tval, int32_t* __restrict__ out_in, double* __restrict__ out_val) {
    __shared__ int64_t tile[ROW_TILE];
    const unsigned nl = *long_count;
    for (unsigned li = blockIdx.x; li < nl; li += gridDim.x) {
        const int32_t r = long_list[li];
        const int64_t s = row_start[r], t = row_start[r + 1], len = t - s;
        for (int64_t e0 = s; e0 < t; e0 += (int64_t)blockDim.x * 8) {
            int64_t mykey[8];
            int64_t rank[8];
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int64_t e = e0 + threadIdx.x + (int64_t)k * blockDim.x;
                mykey[k] = e < t ? tkey[e] : INT64_MAX;
                rank[k] = 0;
            }
            for (int64_t q0 = 0; q0 < len; q0 += ROW_TILE) {
                const int64_t m = len - q0 < ROW_TILE ? len - q0 : ROW_TILE;
                __syncthreads();
                for (int64_t q = threadIdx.x; q < m; q += blockDim.x) tile[q] = tkey[s + q0 + q];
                __syncthreads();
                for (int64_t q = 0; q < m; q++) {
                    const int64_t kq = tile[q];
#pragma unroll
                    for (int k = 0; k < 8; k++) rank[k] += kq < mykey[k];
                }
            }
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int64_t e = e0 + threadIdx.x + (int64_t)k * blockDim.x;
                if (e < t) {
                    out_in[s + rank[k]] = (int32_t)(mykey[k] >> 32);
                    out_val[s + rank[k]] = tval[e];
                }
            }
        }
        __syncthreads();
    }
}

__global__ void make_keys(const int32_t* raw_in, int64_t n, int64_t* skey) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        skey[k] = ((int64_t)raw_in[k] << 32) | (int64_t)(uint32_t)k;
}

// numpy's pairwise summation for n <= 128 (used by add.reduce / reduceat):
// a sequential sum from -0.0 below 8 terms, else 8 interleaved partial sums.
template <typename At>
__device__ double pw_block(const At& at, int64_t off, int64_t n) {
    if (n < 8) {
        double res = -0.0;
        for (int64_t i = 0; i < n; i++) res = dadd(res, at(off + i));
        return res;
    }
    double r[8];
#pragma unroll
    for (int j = 0; j < 8; j++) r[j] = at(off + j);
    int64_t i = 8;
    for (; i < n - (n % 8); i += 8) {
#pragma unroll
        for (int j = 0; j < 8; j++) r[j] = dadd(r[j], at(off + i + j));
    }
    double res = dadd(dadd(dadd(r[0], r[1]), dadd(r[2], r[3])), dadd(dadd(r[4], r[5]), dadd(r[6], r[7])));
    for (; i < n; i++) res = dadd(res, at(off + i));
    return res;
}

// numpy pairwise_sum: blocks of at most 128 terms, larger ranges split at
// n/2 rounded down to a multiple of 8 (iterative form of the recursion)
template <typename At>
__device__ double pairwise_sum(const At& at, int64_t off, int64_t n) {
    struct Frame {
        int64_t off, n;
        double left;
        int stage;
    };
    Frame stk[48];
    int sp = 0;
    stk[0] = {off, n, 0.0, 0};
    for (;;) {
        Frame& f = stk[sp];
        if (f.n <= 128) {
            double result = pw_block(at, f.off, f.n);
            for (;;) {
                if (sp == 0) return result;
                sp--;
                Frame& p = stk[sp];
                if (p.stage == 1) {
                    p.left = result;
                    p.stage = 2;
                    int64_t n2 = p.n / 2;
                    n2 -= n2 % 8;
                    stk[sp + 1] = {p.off + n2, p.n - n2, 0.0, 0};
                    sp++;
                    break;
                }
                result = dadd(p.left, result);
            }
        } else {
            f.stage = 1;
            int64_t n2 = f.n / 2;
            n2 -= n2 % 8;
            stk[sp + 1] = {f.off, n2, 0.0, 0};
            sp++;
        }
    }
}


// One thread per output cell: merge equal input indices of the cell's sorted
// raw entries with the add.reduceat association, first + pairwise(rest),
// writing (col, value) compactly from the bucket start; count them.
// The sorted raw entries arrive as contiguous (input index, value) arrays
// (the bucket sort gathers them while ranking), so each thread reads its
// row's entries in order instead of chasing a permutation.
struct SortedVal {
    const double* val;
    __device__ __forceinline__ double operator()(int64_t k) const { return val[k]; }
};

__global__ void merge_rows(const int64_t* __restrict__ bptr, const int32_t* __restrict__ s_in,
                           const double* __restrict__ s_val, int64_t n_out, int32_t* __restrict__ tmp_col,
                           double* __restrict__ tmp_val, int64_t* __restrict__ row_nnz) {
    SortedVal at{s_val};
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n_out;
         o += (int64_t)gridDim.x * blockDim.x) {
        int64_t s = bptr[o], t = bptr[o + 1];
        int64_t w = s;
        int64_t g = s;
        while (g < t) {
            int32_t c = s_in[g];
            int64_t h = g + 1;
            while (h < t && s_in[h] == c) h++;
            double v = dadd(at(g), pairwise_sum(at, g + 1, h - g - 1));
            tmp_col[w] = c;
            tmp_val[w] = v;
            w++;
            g = h;
        }
        row_nnz[o] = w - s;
    }
}

__global__ void compact_rows(const int64_t* __restrict__ bptr, const int64_t* __restrict__ row_ptr,
                             const int32_t* __restrict__ tmp_col, const double* __restrict__ tmp_val,
                             int64_t n_out, int32_t* __restrict__ col, double* __restrict__ val) {
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n_out;
         o += (int64_t)gridDim.x * blockDim.x) {
        int64_t s = bptr[o], d = row_ptr[o], n = row_ptr[o + 1] - d;
        for (int64_t k = 0; k < n; k++) {
            col[d + k] = tmp_col[s + k];
            val[d + k] = tmp_val[s + k];
        }
    }
}

// Bins of a static grid with bounding box bb: square, sized so that a bin
// holds about one edge along the boundary; at most 1024 a side.
Bins static_bins(const double* bb, int64_t nedges) {
    const double ex = bb[2] - bb[0], ey = bb[3] - bb[1];
    const double ext = ex > ey ? ex : ey;
    int64_t side = nedges / 8;
    if (side < 8) side = 8;
    if (side > 1024) side = 1024;
    const double hbin = ext > 0 && std::isfinite(ext) ? ext / (double)side : 1.0;
    Bins b;
    b.ox = bb[0];
    b.oy = bb[1];
    b.inv_h = 1.0 / hbin;
    b.nbx = (int)std::min<double>(1024.0, std::max(1.0, std::ceil(ex / hbin)));
    b.nby = (int)std::min<double>(1024.0, std::max(1.0, std::ceil(ey / hbin)));
    if (!std::isfinite(ex) || !std::isfinite(ey)) {
        b.nbx = 1;
        b.nby = 1;
    }
    b.ptr = nullptr;
    b.items = nullptr;
    return b;
}

// Batch-wide arrays of the static grids' preparation (PrepGrid)
struct StaticBatch {
    PrepGrid* grids = nullptr;  // [2G]
    Edge* edges = nullptr;
    unsigned* counts = nullptr;
    int64_t* ptr64 = nullptr;
    int32_t* ptr32 = nullptr;
    int32_t* items = nullptr;
    double* bbox_part = nullptr;
    void free(cudaStream_t s) {
        dfree(grids, s);
        dfree(edges, s);
        dfree(counts, s);
        dfree(ptr64, s);
        dfree(ptr32, s);
        dfree(items, s);
        dfree(bbox_part, s);
        *this = StaticBatch();
    }
};

}  // namespace

int cell_area_2d(const double* x, const double* y, int64_t nx, int64_t ny, double* area,
                 cudaStream_t s) {
    int64_t n = (nx - 1) * (ny - 1);
    if (n <= 0) return RG_OK;
    cell_area_kernel<<<grid_for(n, 256), 256, 0, s>>>(x, y, nx, ny, area);
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

// Seat lookup for points (the locator entry point): method 0 brute, 1 secant
__global__ void locate_points_kernel(Grid g, const double* px, const double* py, int64_t n,
                                     int method, int64_t* oi, int64_t* oj) {
    int lane = threadIdx.x & 31;
    int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (k >= n) return;
    double x = px[k], y = py[k];
    int64_t i = MAXSIZE, j = MAXSIZE;
    int ok = 0;
    if (method == 1) {
        if (lane == 0) ok = locate_secant(g, x, y, &i, &j);
        ok = __shfl_sync(0xffffffffu, ok, 0);
    }
    if (!ok) locate_brute_warp(g, x, y, &i, &j);
    if (lane == 0) {
        oi[k] = i;
        oj[k] = j;
    }
}

int locate_2d_exact(const double* x, const double* y, int64_t nx, int64_t ny, const double* px,
                    const double* py, int64_t n, int method, int64_t* oi, int64_t* oj,
                    cudaStream_t s) {
    if (n <= 0) return RG_OK;
    locate_points_kernel<<<grid_for(n * 32, 128), 128, 0, s>>>(Grid{x, y, nx, ny}, px, py, n, method,
                                                               oi, oj);
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

std::atomic<int64_t> g_sweep_chunk{32};
// the walk kernel keeps 8 blocks of 64 threads per SM: 152 x 512 threads
constexpr int64_t kTargetChunks = 152 * 512;
constexpr int64_t kMinChunk = 4;

namespace {

// The walk failures a grid's error word records, as a status (message set).
int walk_status(unsigned fl) {
    if (fl & (FLAG_WALK_CAP | FLAG_SEAT_OUTSIDE)) {
        set_error("conservative sweep: %s",
                  (fl & FLAG_WALK_CAP) ? "a grid line exceeded its step cap (degenerate grids?)"
                                       : "a grid line starting inside the grid boundary could "
                                         "not be located in any cell");
        return RG_ERR_WALK;
    }
    return RG_OK;
}

template <typename T>
int upload(T** d, const std::vector<T>& h, cudaStream_t s) {
    RG_TRY(dalloc(d, h.size(), s));
    RG_TRY(small_to_device(*d, h.data(), sizeof(T) * h.size(), s));
    return RG_OK;
}

// One thread per line over all lines of the batch, count then write
// (synchronises once).  fl receives every grid's error word.
int sweep_lines(const Batch& B, int64_t lines, const Seat* seats, int64_t* total_dev, cudaStream_t s,
                int32_t** raw_in, int32_t** raw_out, double** raw_val, int64_t* nraw_out, std::vector<unsigned>& fl) {
    int64_t *counts = nullptr, *offsets = nullptr;
    int st = RG_OK;
    do {
        if ((st = dalloc(&counts, (size_t)lines + 1, s))) break;
        if ((st = dalloc(&offsets, (size_t)lines + 1, s))) break;
        walk_kernel<false><<<grid_for(lines, 64), 64, 0, s>>>(B, seats, counts, nullptr, nullptr, nullptr, nullptr);
        zero_async(counts + lines, sizeof(int64_t), s);
        if ((st = exclusive_scan_i64(counts, offsets, lines + 1, total_dev, s))) break;
        int64_t nraw = 0;
        small_to_host(&nraw, total_dev, sizeof(int64_t), s);
        small_to_host(fl.data(), B.flags, sizeof(unsigned) * fl.size(), s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("conservative sweep (count walk): %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }
        if (nraw >= (int64_t)UINT32_MAX) {
            set_error("conservative sweep: %lld raw entries exceed 2^32", (long long)nraw);
            st = RG_ERR_UNSUPPORTED;
            break;
        }
        if ((st = dalloc(raw_in, (size_t)nraw, s))) break;
        if ((st = dalloc(raw_out, (size_t)nraw, s))) break;
        if ((st = dalloc(raw_val, (size_t)nraw, s))) break;
        walk_kernel<true><<<grid_for(lines, 64), 64, 0, s>>>(B, seats, nullptr, offsets, *raw_in, *raw_out, *raw_val);
        *nraw_out = nraw;
    } while (0);
    dfree(counts, s);
    dfree(offsets, s);
    return st;
}

// The triples ordered by output row straight from the chunks' slots
// (slot_count_rows, slot_scatter_rows, rank_rows): row_start[n_rows + 1] and
// the rows' input cells and values.
struct SortedRows {
    int64_t n_rows = 0;
    int64_t* row_start = nullptr;
    int32_t* in = nullptr;
    double* val = nullptr;
};

// Chunked walk over all lines of the batch (see chunk_walk_kernel), its
// triples left in output-row order in *rows.  Sets *nraw_out to -1 (and
// frees everything) when a chunk needed more slots than it was given or the
// slots would not fit; fl receives every grid's error word.

int sweep_chunked(Batch& B, const std::vector<SweepParams>& P, const std::vector<double>& bbox_h,
                  const Seat* seats, int64_t lines, int64_t* total_dev, cudaStream_t s, int64_t* nraw_out,
                  std::vector<unsigned>& fl, ChunkPlan** plans_dev, int64_t** chunk_base_dev, SortedRows* rows) {
    const int G = B.G;
    // sweep segments per chunk: rg_set_sweep_chunk (default 32), the
    // RG_SWEEP_CHUNK environment variable overriding it (0 walks whole lines)
    int64_t ch = g_sweep_chunk.load();
    if (const char* env = getenv("RG_SWEEP_CHUNK")) {
        ch = atoll(env);
    } else if (ch > kMinChunk) {
        // Small batches: shorter chunks, so that the walk still has about
        // kTargetChunks threads (each chunk is one thread's sequential walk;
        // a 128^2 pair in chunks of 32 segments keeps 2,000 threads busy
        // for 0.7 ms).  Every chunk length gives the same triples in the
        // same order.
        int64_t segments = 0;
        for (int g = 0; g < G; g++)
            for (int f = 0; f < 4; f++) segments += P[g].fam[f].lines * (P[g].fam[f].len - 1);
        const int64_t fit = (segments + kTargetChunks - 1) / kTargetChunks;
        ch = std::min<int64_t>(ch, std::max<int64_t>(kMinChunk, fit));
    }
    *nraw_out = -1;
    if (ch <= 0) return RG_OK;
    // fault injection for tests: RG_FAULT_CHUNK_SLOTS caps the triple slots
    // a chunk gets, so chunks overflow and the build takes its recovery path
    // (whole-line walks, which count exactly); the weights do not change
    int64_t slot_cap = INT64_MAX;
    if (const char* env = getenv("RG_FAULT_CHUNK_SLOTS")) slot_cap = std::max<int64_t>(1, atoll(env));
    std::vector<ChunkPlan> C((size_t)G);
    std::vector<int64_t> chunk_base((size_t)G + 1, 0);
    int64_t chunks = 0, slots = 0;
    for (int g = 0; g < G; g++) {
        ChunkPlan& c = C[g];
        memset(&c, 0, sizeof(c));
        c.ch = ch;
        chunk_base[g] = chunks;
        const double* bb = bbox_h.data() + 8 * g;
        for (int f = 0; f < 4; f++) {
            const Family& F = P[g].fam[f];
            const Static& S = P[g].st[F.st];
            const double* bs = F.sweep_input ? bb : bb + 4;  // sweep grid's box
            const double* bt = F.sweep_input ? bb + 4 : bb;  // static grid's box
            double seg = fmax(bs[2] - bs[0], bs[3] - bs[1]) / (double)(F.len - 1 > 0 ? F.len - 1 : 1);
            double dens = fmax((double)S.ncx / fmax(bt[2] - bt[0], 1e-300), (double)S.ncy / fmax(bt[3] - bt[1], 1e-300));
            double cross = 2.0 * ceil(1.5 * seg * dens) + 2.0;
            if (!(cross < 1e6)) cross = 1e6;
            c.nc[f] = (F.len - 1 + ch - 1) / ch;
            c.chunk_base[f] = chunks;
            c.cap[f] = std::min<int64_t>(2 * ch * (1 + (int64_t)cross) + 32, slot_cap);
            c.slot_base[f] = slots;
            chunks += F.lines * c.nc[f];
            slots += F.lines * c.nc[f] * c.cap[f];
        }
        c.chunk_base[4] = chunks;
    }
    chunk_base[G] = chunks;
    if (slots * 16 > (int64_t)24 << 30 || slots >= (int64_t)1 << 40) return RG_OK;  // too big: walk lines

    WalkState *starts = nullptr, *ends = nullptr;
    int64_t *counts = nullptr, *offsets = nullptr;
    int32_t *s_in = nullptr, *s_out = nullptr;
    double* s_val = nullptr;
    unsigned long long* n_rep = nullptr;
    int st = RG_OK;
    bool overflow = false;
    do {
        if ((st = upload(plans_dev, C, s))) break;
        if ((st = upload(chunk_base_dev, chunk_base, s))) break;
        B.C = *plans_dev;
        B.chunk_base = *chunk_base_dev;
        if ((st = dalloc(&starts, (size_t)chunks, s))) break;
        if ((st = dalloc(&ends, (size_t)chunks, s))) break;
        if ((st = dalloc(&counts, (size_t)chunks + 1, s))) break;
        if ((st = dalloc(&offsets, (size_t)chunks + 1, s))) break;
        if ((st = dalloc(&n_rep, 2, s))) break;  // chunks repaired, next chunk of the walk
        if ((st = dalloc(&s_in, (size_t)slots, s))) break;
        if ((st = dalloc(&s_out, (size_t)slots, s))) break;
        if ((st = dalloc(&s_val, (size_t)slots, s))) break;
        zero_async(n_rep, 2 * sizeof(unsigned long long), s);
        chunk_seat_kernel<<<grid_for(chunks, 128), 128, 0, s>>>(B, seats, starts);
        {
            // resident blocks only: 8 blocks of 64 threads per SM
            const unsigned blocks = std::min<unsigned>(grid_for(chunks, 64), 152u * 8u);
            chunk_walk_kernel<<<blocks, 64, 0, s>>>(B, starts, ends, counts, s_in, s_out, s_val, n_rep + 1);
        }
        chunk_repair_kernel<<<grid_for(lines, 64), 64, 0, s>>>(B, starts, ends, counts, s_in, s_out, s_val, n_rep);
        zero_async(counts + chunks, sizeof(int64_t), s);
        if ((st = exclusive_scan_i64(counts, offsets, chunks + 1, total_dev, s))) break;
        int64_t nraw = 0;
        small_to_host(&nraw, total_dev, sizeof(int64_t), s);
        small_to_host(fl.data(), B.flags, sizeof(unsigned) * fl.size(), s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("conservative sweep (chunked walk): %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }
        bool cap = false;
        for (unsigned f : fl) cap = cap || (f & FLAG_CAPACITY);
        if (cap) {
            overflow = true;
            zero_async(B.flags, sizeof(unsigned) * fl.size(), s);
            break;
        }
        if (nraw >= (int64_t)UINT32_MAX) {
            set_error("conservative sweep: %lld raw entries exceed 2^32", (long long)nraw);
            st = RG_ERR_UNSUPPORTED;
            break;
        }
        {
            // order the triples by output row from the slots
            const int64_t nr = rows->n_rows;
            unsigned *rowc = nullptr, *long_count = nullptr;
            int64_t* tkey = nullptr;
            double* tval = nullptr;
            int32_t* long_list = nullptr;
            do {
                if ((st = dalloc(&rows->row_start, (size_t)nr + 1, s))) break;
                if ((st = dalloc(&rows->in, (size_t)std::max<int64_t>(nraw, 1), s))) break;
                if ((st = dalloc(&rows->val, (size_t)std::max<int64_t>(nraw, 1), s))) break;
                if ((st = dalloc(&rowc, (size_t)nr + 1, s))) break;
                if ((st = dalloc(&long_count, 1, s))) break;
                if ((st = dalloc(&long_list, (size_t)std::max<int64_t>(nr, 1), s))) break;
                if ((st = dalloc(&tkey, (size_t)std::max<int64_t>(nraw, 1), s))) break;
                if ((st = dalloc(&tval, (size_t)std::max<int64_t>(nraw, 1), s))) break;
                zero_async(rowc, sizeof(unsigned) * (nr + 1), s);
                zero_async(long_count, sizeof(unsigned), s);
                slot_count_rows<<<grid_for(chunks * 32, 256), 256, 0, s>>>(B, counts, s_out, rowc);
                if ((st = exclusive_scan_u32_to_i64(rowc, rows->row_start, nr + 1, nullptr, s))) break;
                zero_async(rowc, sizeof(unsigned) * (nr + 1), s);
                slot_scatter_rows<<<grid_for(chunks * 32, 256), 256, 0, s>>>(B, counts, offsets, s_in, s_out, s_val,
                                                                           rows->row_start, rowc, tkey, tval);
                const unsigned gr = grid_for(nr * 32, 256) > 16384 ? 16384 : grid_for(nr * 32, 256);
                rank_rows<<<gr, 256, 0, s>>>(rows->row_start, nr, tkey, tval, rows->in, rows->val, long_list,
                                             long_count);
                rank_rows_long<<<1024, 256, 0, s>>>(rows->row_start, long_list, long_count, tkey, tval, rows->in,
                                                    rows->val);
            } while (0);
            dfree(rowc, s);
            dfree(long_count, s);
            dfree(long_list, s);
            dfree(tkey, s);
            dfree(tval, s);
            if (st) break;
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error("conservative sweep (compaction): %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }
        *nraw_out = nraw;
    } while (0);
    dfree(starts, s);
    dfree(ends, s);
    dfree(counts, s);
    dfree(offsets, s);
    dfree(n_rep, s);
    dfree(s_in, s);
    dfree(s_out, s);
    dfree(s_val, s);
    if (overflow) *nraw_out = -1;
    return st;
}

// Per-grid sizes of the merged CSR: nnz_base[g] = row_ptr[out_base[g]].
__global__ void nnz_bases(const int64_t* __restrict__ row_ptr, const int64_t* __restrict__ out_base, int G,
                          int64_t* __restrict__ nnz_base) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g <= G; g += gridDim.x * blockDim.x)
        nnz_base[g] = row_ptr[out_base[g]];
}

// Copy every grid's rows and entries of the merged CSR to its own arrays.
__global__ void split_rows(const int64_t* __restrict__ row_ptr, const int64_t* __restrict__ out_base,
                           const int64_t* __restrict__ nnz_base, int G, int64_t* const* __restrict__ dst_row_ptr) {
    const int64_t n = out_base[G];
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const int g = pair_of(out_base, G, r);
        const int64_t local = r - out_base[g];
        dst_row_ptr[g][local] = row_ptr[r] - nnz_base[g];
        if (r + 1 == out_base[g + 1]) dst_row_ptr[g][local + 1] = row_ptr[r + 1] - nnz_base[g];
    }
}
__global__ void split_entries(const int32_t* __restrict__ col, const double* __restrict__ val,
                              const int64_t* __restrict__ nnz_base, int G, int32_t* const* __restrict__ dst_col,
                              double* const* __restrict__ dst_val) {
    const int64_t n = nnz_base[G];
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int g = pair_of(nnz_base, G, k);
        const int64_t local = k - nnz_base[g];
        dst_col[g][local] = col[k];
        dst_val[g][local] = val[k];
    }
}

}  // namespace

// Conservative weights of G grid pairs in one pass: every stage runs once
// over all pairs (their lines, chunks and output rows concatenated), and the
// batch synchronises with the host five times whatever G is.  W[g] receives
// pair g's CSR when status[g] is RG_OK; a pair whose sweep fails (degenerate
// grids) gets its error in status[g] and leaves the others unaffected.
int build_batch(const PairSpec* pairs, int G, cudaStream_t s, rg_weights_s** W, int* status) {
    RG_CHECK(G >= 1, RG_ERR_ARG, "conservative batch: no grid pairs");
    std::vector<int64_t> in_base((size_t)G + 1, 0), out_base((size_t)G + 1, 0), line_base((size_t)G + 1, 0);
    for (int g = 0; g < G; g++) {
        const PairSpec& q = pairs[g];
        RG_CHECK(q.nxi >= 2 && q.nyi >= 2 && q.nxo >= 2 && q.nyo >= 2, RG_ERR_ARG,
                 "conservative 2D grids need at least 2 vertices per axis");
        const int64_t n_in = (q.nxi - 1) * (q.nyi - 1), n_out = (q.nxo - 1) * (q.nyo - 1);
        in_base[g + 1] = in_base[g] + n_in;
        out_base[g + 1] = out_base[g] + n_out;
        // lines of the four families: output rows/columns, then input rows/columns
        line_base[g + 1] = line_base[g] + q.nyo + q.nxo + q.nyi + q.nxi;
        status[g] = RG_OK;
    }
    RG_CHECK(in_base[G] < INT32_MAX && out_base[G] < INT32_MAX, RG_ERR_UNSUPPORTED,
             "grids above 2^31 cells (in a batch, in total) are not supported");
    const int64_t lines = line_base[G], n_out_all = out_base[G];

    int st = RG_OK;
    double* area_in = nullptr;
    double* bbox_d = nullptr;
    StaticBatch SB;
    int64_t* totals = nullptr;
    SweepParams* P_dev = nullptr;
    int64_t *line_base_dev = nullptr, *out_base_dev = nullptr, *chunk_base_dev = nullptr;
    ChunkPlan* plans_dev = nullptr;
    Seat* seats = nullptr;
    int64_t* total_dev = nullptr;
    unsigned* flags = nullptr;
    int32_t *raw_in = nullptr, *raw_out = nullptr, *sorted_in = nullptr;
    double* sorted_val = nullptr;
    double* raw_val = nullptr;
    int64_t* skey = nullptr;
    int64_t* bucket_ptr = nullptr;
    uint32_t* perm = nullptr;
    int32_t* tmp_col = nullptr;
    double* tmp_val = nullptr;
    int64_t* row_nnz = nullptr;
    int64_t* row_ptr = nullptr;
    int32_t* col = nullptr;
    double* val = nullptr;
    int64_t* nnz_base_dev = nullptr;
    void** dst_dev = nullptr;  // [3G]: row_ptr, col, val pointers of every grid

    do {
        // static grids: the input and the output grid of every pair.  Areas
        // of the input cells, bounding boxes and boundary edges of all grids
        // (sync 1 reads the boxes)
        const int NG = 2 * G;
        std::vector<PrepGrid> PG((size_t)NG);
        int64_t nedges_all = 0, max_verts = 0;
        for (int k = 0; k < NG; k++) {
            const PairSpec& q = pairs[k >> 1];
            PrepGrid& r = PG[k];
            memset(&r, 0, sizeof(PrepGrid));
            r.g = (k & 1) ? Grid{q.xo, q.yo, q.nxo, q.nyo} : Grid{q.xi, q.yi, q.nxi, q.nyi};
            r.cell_base = (k & 1) ? 0 : in_base[k >> 1];
            r.edge_base = nedges_all;
            nedges_all += 2 * (r.g.nx - 1) + 2 * (r.g.ny - 1);
            max_verts = std::max(max_verts, r.g.nx * r.g.ny);
        }
        // blocks per grid for the boxes: about 16 vertices a thread, 1..256
        const int nparts = (int)std::min<int64_t>(256, std::max<int64_t>(1, (max_verts + 4095) / 4096));
        if ((st = upload(&SB.grids, PG, s))) break;
        if ((st = dalloc(&area_in, (size_t)in_base[G], s))) break;
        if ((st = dalloc(&bbox_d, (size_t)4 * NG, s))) break;
        if ((st = dalloc(&SB.bbox_part, (size_t)4 * NG * nparts, s))) break;
        if ((st = dalloc(&SB.edges, (size_t)nedges_all, s))) break;
        cell_area_batch<<<grid_for(in_base[G], 256), 256, 0, s>>>(SB.grids, G, in_base[G], area_in);
        bbox_partial_batch<<<(unsigned)(NG * nparts), 256, 0, s>>>(SB.grids, nparts, SB.bbox_part);
        bbox_combine_batch<<<grid_for((int64_t)NG * 32, 128), 128, 0, s>>>(SB.bbox_part, nparts, NG, bbox_d);
        boundary_edges_batch<<<grid_for(nedges_all, 128), 128, 0, s>>>(SB.grids, NG, nedges_all, SB.edges);
        std::vector<double> bbox_h((size_t)4 * NG);
        small_to_host(bbox_h.data(), bbox_d, sizeof(double) * 4 * NG, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("conservative build: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }

        // bins of every static grid: count the edges of each bin, one scan
        // over the slots of all grids (sync 2 reads the item total), file
        int64_t nslots = 0;
        for (int k = 0; k < NG; k++) {
            PrepGrid& r = PG[k];
            r.b = static_bins(bbox_h.data() + 4 * k, 2 * (r.g.nx - 1) + 2 * (r.g.ny - 1));
            r.bin_base = nslots;
            nslots += (int64_t)r.b.nbx * r.b.nby + 1;
        }
        if ((st = small_to_device(SB.grids, PG.data(), sizeof(PrepGrid) * PG.size(), s))) break;
        if ((st = dalloc(&totals, 1, s))) break;
        if ((st = dalloc(&SB.counts, (size_t)nslots, s))) break;
        if ((st = dalloc(&SB.ptr64, (size_t)nslots, s))) break;
        if ((st = dalloc(&SB.ptr32, (size_t)nslots, s))) break;
        if ((st = zero_async(SB.counts, sizeof(unsigned) * nslots, s))) break;
        bin_edges_batch<false><<<grid_for(nedges_all, 128), 128, 0, s>>>(SB.grids, NG, SB.edges, nedges_all,
                                                                          SB.counts, nullptr, nullptr);
        if ((st = exclusive_scan_u32_to_i64(SB.counts, SB.ptr64, nslots, totals, s))) break;
        int64_t nitems = 0;
        small_to_host(&nitems, totals, sizeof(int64_t), s);
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("conservative build: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }
        if (nitems >= (int64_t)INT32_MAX) {
            set_error("conservative build: %lld binned boundary edges exceed 2^31", (long long)nitems);
            st = RG_ERR_UNSUPPORTED;
            break;
        }
        if ((st = dalloc(&SB.items, (size_t)nitems, s))) break;
        if ((st = zero_async(SB.counts, sizeof(unsigned) * nslots, s))) break;
        bin_edges_batch<true><<<grid_for(nedges_all, 128), 128, 0, s>>>(SB.grids, NG, SB.edges, nedges_all,
                                                                         SB.counts, SB.items, SB.ptr64);
        i64_to_i32<<<grid_for(nslots, 256), 256, 0, s>>>(SB.ptr64, SB.ptr32, nslots);
        e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error("conservative build (static grids): %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }
        std::vector<SweepParams> P((size_t)G);
        for (int g = 0; g < G; g++) {
            memset(&P[g], 0, sizeof(SweepParams));
            for (int side = 0; side < 2; side++) {
                const PrepGrid& r = PG[2 * g + side];
                const double* bb = bbox_h.data() + 4 * (2 * g + side);
                Static& S = P[g].st[side];
                S.g = r.g;
                S.ncx = r.g.nx - 1;
                S.ncy = r.g.ny - 1;
                S.blx = bb[0];
                S.bly = bb[1];
                S.bux = bb[2];
                S.buy = bb[3];
                S.nbound = 2 * S.ncx + 2 * S.ncy;
                S.edges = SB.edges + r.edge_base;
                S.bins = r.b;
                S.bins.ptr = SB.ptr32 + r.bin_base;
                S.bins.items = SB.items;
            }
        }

        // sweep families in upstream order: sweep output (axis 0, 1), sweep
        // input (axis 0, 1); line bases global across the batch
        for (int g = 0; g < G; g++) {
            const PairSpec& q = pairs[g];
            int64_t base = line_base[g];
            for (int k = 0; k < 4; k++) {
                Family& F = P[g].fam[k];
                F.sweep_input = k >= 2;
                F.axis = k & 1;
                F.sweep = F.sweep_input ? Grid{q.xi, q.yi, q.nxi, q.nyi} : Grid{q.xo, q.yo, q.nxo, q.nyo};
                F.st = F.sweep_input ? 1 : 0;
                F.transposed = F.axis == 0;
                F.lines = F.axis == 0 ? F.sweep.ny : F.sweep.nx;
                F.len = F.axis == 0 ? F.sweep.nx : F.sweep.ny;
                F.line_base = base;
                base += F.lines;
            }
            P[g].total_lines = base;
            P[g].area_in = area_in + in_base[g];
            P[g].w_in = q.w_in;
            P[g].ncy_in = q.nyi - 1;
            P[g].ncy_out = q.nyo - 1;
        }
        if ((st = upload(&P_dev, P, s))) break;
        if ((st = upload(&line_base_dev, line_base, s))) break;
        if ((st = upload(&out_base_dev, out_base, s))) break;
        if ((st = dalloc(&flags, (size_t)G, s))) break;
        if ((st = dalloc(&total_dev, 1, s))) break;
        zero_async(flags, sizeof(unsigned) * G, s);
        Batch B;
        B.P = P_dev;
        B.C = nullptr;
        B.line_base = line_base_dev;
        B.chunk_base = nullptr;
        B.out_base = out_base_dev;
        B.flags = flags;
        B.G = G;

        // seats and the sweep (sync 3)
        if ((st = dalloc(&seats, (size_t)lines, s))) break;
        seat_kernel<<<grid_for(lines * 32, 128), 128, 0, s>>>(B, seats);
        std::vector<unsigned> fl((size_t)G, 0u);
        int64_t nraw = 0;
        SortedRows rows;
        rows.n_rows = n_out_all;
        st = sweep_chunked(B, P, bbox_h, seats, lines, total_dev, s, &nraw, fl, &plans_dev, &chunk_base_dev,
                           &rows);
        bucket_ptr = rows.row_start;
        sorted_in = rows.in;
        sorted_val = rows.val;
        if (st) break;
        if (nraw < 0) {
            // a chunk overflowed its slots: walk whole lines instead
            if ((st = sweep_lines(B, lines, seats, total_dev, s, &raw_in, &raw_out, &raw_val, &nraw, fl))) break;
        }
        for (int g = 0; g < G; g++) status[g] = walk_status(fl[g]);

        // merge: the triples in output-row order (sync 4 for the entry count;
        // the per-grid sizes come with it).  The chunked walk orders them from
        // its slots; otherwise one bucket sort over the output rows of the
        // whole batch, which also lays the entries' input indices and values
        // out in sorted order, so the merge reads them contiguously.
        if (bucket_ptr == nullptr) {
            if ((st = dalloc(&skey, (size_t)nraw, s))) break;
            if ((st = dalloc(&bucket_ptr, (size_t)n_out_all + 1, s))) break;
            if ((st = dalloc(&perm, (size_t)nraw, s))) break;
            if (nraw > 0)
                make_keys<<<grid_for(nraw, 256) > 8192 ? 8192 : grid_for(nraw, 256), 256, 0, s>>>(raw_in, nraw,
                                                                                                   skey);
            if ((st = dalloc(&sorted_in, (size_t)nraw, s))) break;
            if ((st = dalloc(&sorted_val, (size_t)nraw, s))) break;
            if ((st = bucket_sort(raw_out, skey, nraw, n_out_all, bucket_ptr, perm, flags, s, raw_val, sorted_in,
                                  sorted_val)))
                break;
            dfree(skey, s);
            skey = nullptr;
            dfree(raw_in, s);
            dfree(raw_out, s);
            dfree(raw_val, s);
            raw_in = raw_out = nullptr;
            raw_val = nullptr;
        }
        if ((st = dalloc(&tmp_col, (size_t)nraw, s))) break;
        if ((st = dalloc(&tmp_val, (size_t)nraw, s))) break;
        if ((st = dalloc(&row_nnz, (size_t)n_out_all + 1, s))) break;
        zero_async(row_nnz + n_out_all, sizeof(int64_t), s);
        merge_rows<<<grid_for(n_out_all, 128), 128, 0, s>>>(bucket_ptr, sorted_in, sorted_val, n_out_all, tmp_col,
                                                            tmp_val, row_nnz);
        if ((st = dalloc(&row_ptr, (size_t)n_out_all + 1, s))) break;
        if ((st = exclusive_scan_i64(row_nnz, row_ptr, n_out_all + 1, total_dev, s))) break;
        if ((st = dalloc(&nnz_base_dev, (size_t)G + 1, s))) break;
        nnz_bases<<<grid_for(G + 1, 128), 128, 0, s>>>(row_ptr, out_base_dev, G, nnz_base_dev);
        std::vector<int64_t> nnz_base((size_t)G + 1, 0);
        small_to_host(nnz_base.data(), nnz_base_dev, sizeof(int64_t) * (G + 1), s);
        std::vector<unsigned> fl2((size_t)G, 0u);
        small_to_host(fl2.data(), flags, sizeof(unsigned) * G, s);
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("conservative build (merge): %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }
        for (int g = 0; g < G; g++)
            if (status[g] == RG_OK && (fl2[g] & FLAG_CAPACITY)) {
                set_error("conservative sweep: the write walk disagreed with the count walk");
                status[g] = RG_ERR_WALK;
            }
        const int64_t nnz = nnz_base[G];
        if ((st = dalloc(&col, (size_t)nnz, s))) break;
        if ((st = dalloc(&val, (size_t)nnz, s))) break;
        compact_rows<<<grid_for(n_out_all, 128), 128, 0, s>>>(bucket_ptr, row_ptr, tmp_col, tmp_val, n_out_all, col,
                                                              val);
        e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error("conservative build: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }

        // hand every grid its CSR: a single pair takes the arrays as they
        // are, several get their own copies (no synchronisation)
        auto fill_handle = [&](int g) {
            const PairSpec& q = pairs[g];
            W[g]->n_in = in_base[g + 1] - in_base[g];
            W[g]->n_out = out_base[g + 1] - out_base[g];
            W[g]->nnz = nnz_base[g + 1] - nnz_base[g];
            W[g]->out_shape0 = q.nxo - 1;
            W[g]->out_shape1 = q.nyo - 1;
            W[g]->in_shape0 = q.nxi - 1;
            W[g]->in_shape1 = q.nyi - 1;
        };
        if (G == 1) {
            W[0]->row_ptr = row_ptr;
            W[0]->col = col;
            W[0]->val = val;
            fill_handle(0);
            row_ptr = nullptr;
            col = nullptr;
            val = nullptr;
            break;
        }
        std::vector<void*> dst((size_t)3 * G, nullptr);
        for (int g = 0; g < G && st == RG_OK; g++) {
            if (status[g] != RG_OK) continue;
            fill_handle(g);
            if ((st = dalloc(&W[g]->row_ptr, (size_t)W[g]->n_out + 1, s))) break;
            if ((st = dalloc(&W[g]->col, (size_t)W[g]->nnz, s))) break;
            if ((st = dalloc(&W[g]->val, (size_t)W[g]->nnz, s))) break;
            dst[g] = W[g]->row_ptr;
            dst[G + g] = W[g]->col;
            dst[2 * G + g] = W[g]->val;
        }
        if (st) break;
        // grids that failed get scratch destinations: their rows are copied and dropped
        int64_t max_rows = 0, max_nnz = 0;
        for (int g = 0; g < G; g++)
            if (dst[g] == nullptr) {
                max_rows = std::max(max_rows, out_base[g + 1] - out_base[g] + 1);
                max_nnz = std::max(max_nnz, nnz_base[g + 1] - nnz_base[g]);
            }
        int64_t* junk_rows = nullptr;
        int32_t* junk_col = nullptr;
        double* junk_val = nullptr;
        if (max_rows > 0) {
            if ((st = dalloc(&junk_rows, (size_t)max_rows, s))) break;
            if ((st = dalloc(&junk_col, (size_t)std::max<int64_t>(max_nnz, 1), s))) break;
            if ((st = dalloc(&junk_val, (size_t)std::max<int64_t>(max_nnz, 1), s))) break;
            for (int g = 0; g < G; g++)
                if (dst[g] == nullptr) {
                    dst[g] = junk_rows;
                    dst[G + g] = junk_col;
                    dst[2 * G + g] = junk_val;
                }
        }
        if ((st = upload(&dst_dev, dst, s))) break;
        split_rows<<<grid_for(n_out_all, 256) > 8192 ? 8192 : grid_for(n_out_all, 256), 256, 0, s>>>(
            row_ptr, out_base_dev, nnz_base_dev, G, (int64_t* const*)dst_dev);
        if (nnz > 0)
            split_entries<<<grid_for(nnz, 256) > 8192 ? 8192 : grid_for(nnz, 256), 256, 0, s>>>(
                col, val, nnz_base_dev, G, (int32_t* const*)(dst_dev + G), (double* const*)(dst_dev + 2 * G));
        dfree(junk_rows, s);
        dfree(junk_col, s);
        dfree(junk_val, s);
        e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error("conservative build (split): %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }
#ifdef RG_DEBUG
        unsigned dbg = 0;
        const unsigned zero = 0;
        cudaMemcpyFromSymbolAsync(&dbg, g_debug_flags, sizeof(unsigned), 0, cudaMemcpyDeviceToHost, s);
        cudaMemcpyToSymbolAsync(g_debug_flags, &zero, sizeof(unsigned), 0, cudaMemcpyHostToDevice, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) {
            set_error("conservative build (debug flags): %s", cudaGetErrorString(cudaGetLastError()));
            st = RG_ERR_CUDA;
            break;
        }
        if (dbg & FLAG_BOUNDS) {
            set_error("conservative build: debug bounds check: a grid read fell outside its array");
            for (int g = 0; g < G; g++) status[g] = RG_ERR_WALK;
        }
#endif
    } while (0);

    dfree(area_in, s);
    dfree(bbox_d, s);
    SB.free(s);
    dfree(totals, s);
    dfree(P_dev, s);
    dfree(line_base_dev, s);
    dfree(out_base_dev, s);
    dfree(chunk_base_dev, s);
    dfree(plans_dev, s);
    dfree(seats, s);
    dfree(total_dev, s);
    dfree(flags, s);
    dfree(raw_in, s);
    dfree(raw_out, s);
    dfree(raw_val, s);
    dfree(sorted_in, s);
    dfree(sorted_val, s);
    dfree(skey, s);
    dfree(bucket_ptr, s);
    dfree(perm, s);
    dfree(tmp_col, s);
    dfree(tmp_val, s);
    dfree(row_nnz, s);
    dfree(row_ptr, s);
    dfree(col, s);
    dfree(val, s);
    dfree(nnz_base_dev, s);
    dfree(dst_dev, s);
    return st;
}

int build_conservative_2d(const double* xi, const double* yi, int64_t nxi, int64_t nyi,
                          const double* xo, const double* yo, int64_t nxo, int64_t nyo,
                          const double* w_in, cudaStream_t s, rg_weights_s* W) {
    PairSpec q{xi, yi, nxi, nyi, xo, yo, nxo, nyo, w_in};
    int status = RG_OK;
    RG_TRY(build_batch(&q, 1, s, &W, &status));
    return status;
}

}  // namespace rg

extern "C" int rg_set_sweep_chunk(int64_t segments) {
    RG_CHECK(segments >= 0 && segments <= (1 << 20), RG_ERR_ARG, "rg_set_sweep_chunk: %lld out of range",
             (long long)segments);
    rg::g_sweep_chunk.store(segments);
    return RG_OK;
}

