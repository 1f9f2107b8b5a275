// Adjoint of the 2D conservative weights with respect to the output-grid
// vertex coordinates (the backward pass of a differentiable regrid).
//
// A conservative weight is the area of the overlap of input cell i and
// output cell o divided by the area of input cell i (times weights_input[i]):
// the upstream computes it as a sum of contour pieces in its sweep
// (regridding/_weights/_weights_conservative_2d/_weights_conservative_2d.py:
// 752-830).  Its derivative with respect to the output vertices is taken
// here from the same overlap polygon built directly: the output quad is
// clipped against the (convex) input quad edge by edge, every vertex of the
// clipped polygon is typed as an output vertex, an input corner, or the
// crossing of output edge e with input edge f, and its position is computed
// from the original vertices.  The polygon area A = 1/2 sum cross(p_k, p_k+1)
// has dA/dp_k = 1/2 (y_k+1 - y_k-1, x_k-1 - x_k+1); a crossing
// p = a + t (b - a) with input edge c -> d carries it to the output vertices
// a and b as (1 - t) (G + (G.r) n) and t (G + (G.r) n), with r = b - a,
// s = d - c, n = (-s.y, s.x) / cross(r, s).
//
// One thread per output cell: for every stored entry (i, o) it forms
// dL/dw_io = sum_d grad_out[d, o] * values[d, i], multiplies by dw/dA and
// sums the 8 coordinate derivatives of its quad over its entries (in stored
// order) into a per-cell record; a second kernel gives every output vertex
// the sum of its (up to four) cells' corner terms in a fixed order, so the
// gradient is the same bits on every run (no atomics).
#include "common.cuh"

namespace rg {
namespace {

enum : unsigned { FLAG_NONCONVEX = 1u << 8, FLAG_DEGENERATE = 1u << 9 };

// A vertex of the clipped polygon, 40 bytes (two arrays of 12 per thread):
// a crossing keeps its parameter t and the reciprocal of its carriers'
// cross product, from which the gradient pass rebuilds the normal.
struct PV {
    double x, y;
    double t, inv;       // crossing data (kind 2): t along output edge e; 1 / cross(r, s)
    signed char ca, cb;  // carrier lines: 0..3 output edges, 4..7 input edges
    signed char kind;    // 0 output vertex (e), 1 input-only, 2 crossing (e, f)
    signed char e;
};

// float or double values as double (float: exactly, on the integer pipe)
__device__ __forceinline__ double as_double(float v) { return widen(v); }
__device__ __forceinline__ double as_double(double v) { return v; }

__device__ __forceinline__ double cross2(double ax, double ay, double bx, double by) { return ax * by - ay * bx; }

struct Quad {
    double x[4], y[4];
};

__device__ __forceinline__ void load_quad(const double* X, const double* Y, int64_t ny, int64_t i, int64_t j,
                                          Quad& q) {
    // vertex order (i, j), (i+1, j), (i+1, j+1), (i, j+1); edge k runs from
    // vertex k to vertex k+1
    const int64_t v0 = i * ny + j, v1 = (i + 1) * ny + j, v2 = (i + 1) * ny + j + 1, v3 = i * ny + j + 1;
    q.x[0] = __ldg(X + v0), q.y[0] = __ldg(Y + v0);
    q.x[1] = __ldg(X + v1), q.y[1] = __ldg(Y + v1);
    q.x[2] = __ldg(X + v2), q.y[2] = __ldg(Y + v2);
    q.x[3] = __ldg(X + v3), q.y[3] = __ldg(Y + v3);
}

__device__ __forceinline__ double quad_area2(const Quad& q) {
    return cross2(q.x[2] - q.x[0], q.y[2] - q.y[0], q.x[3] - q.x[1], q.y[3] - q.y[1]);
}

__device__ __forceinline__ bool convex(const Quad& q, double orient) {
    for (int k = 0; k < 4; k++) {
        const int a = k, b = (k + 1) & 3, c = (k + 2) & 3;
        if (orient * cross2(q.x[b] - q.x[a], q.y[b] - q.y[a], q.x[c] - q.x[b], q.y[c] - q.y[b]) < 0) return false;
    }
    return true;
}

// the carrier line shared by two consecutive polygon vertices
__device__ __forceinline__ int common_carrier(const PV& p, const PV& q, bool* ok) {
    if (p.ca == q.ca || p.ca == q.cb) return p.ca;
    if (p.cb == q.ca || p.cb == q.cb) return p.cb;
    *ok = false;
    return p.cb;
}

// crossing of carrier line L (output edge L, or input edge L - 4) with input edge f
__device__ PV crossing(const Quad& O, const Quad& C, int L, int f, bool* ok) {
    PV v;
    const double cx = C.x[f], cy = C.y[f];
    const double sx = C.x[(f + 1) & 3] - cx, sy = C.y[(f + 1) & 3] - cy;
    double ax, ay, rx, ry;
    if (L < 4) {
        ax = O.x[L], ay = O.y[L];
        rx = O.x[(L + 1) & 3] - ax, ry = O.y[(L + 1) & 3] - ay;
    } else {
        const int g = L - 4;
        ax = C.x[g], ay = C.y[g];
        rx = C.x[(g + 1) & 3] - ax, ry = C.y[(g + 1) & 3] - ay;
    }
    const double den = cross2(rx, ry, sx, sy);
    double t = 0, inv = 0;
    if (den != 0) {
        inv = 1.0 / den;  // one division serves t and (at the gradient) the normal
        t = cross2(cx - ax, cy - ay, sx, sy) * inv;
    } else {
        *ok = false;
    }
    v.x = ax + t * rx;
    v.y = ay + t * ry;
    v.ca = (signed char)L;
    v.cb = (signed char)(4 + f);
    if (L < 4) {
        v.kind = 2;
        v.e = (signed char)L;
        v.t = t;
        v.inv = inv;
    } else {
        v.kind = 1;
        v.e = -1;
        v.t = v.inv = 0;
    }
    return v;
}

template <typename T>
__global__ void __launch_bounds__(128)
    grad_output_kernel(const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                       const double* __restrict__ val, int64_t n_out, const double* __restrict__ xi,
                       const double* __restrict__ yi, int64_t nyi, const double* __restrict__ xo,
                       const double* __restrict__ yo, int64_t nyo, const double* __restrict__ area_in,
                       const double* __restrict__ w_in, const T* __restrict__ values, const T* __restrict__ gout,
                       int64_t n_in, int64_t stack, double* __restrict__ corner,
                       double* __restrict__ w_check, unsigned* __restrict__ flags) {
    const int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (o >= n_out) return;
    const int64_t ncyo = nyo - 1, ncyi = nyi - 1;
    const int64_t io = o / ncyo, jo = o - io * ncyo;
    Quad O;
    load_quad(xo, yo, nyo, io, jo, O);
    double ax[4] = {0, 0, 0, 0}, ay[4] = {0, 0, 0, 0};
    for (int64_t k = row_ptr[o]; k < row_ptr[o + 1]; k++) {
        const int64_t i = col[k];
        double G = 0;
        for (int64_t d = 0; d < stack; d++) G = fma(as_double(gout[d * n_out + o]), as_double(values[d * n_in + i]), G);
        if (G == 0 && w_check == nullptr) continue;
        const int64_t ii = i / ncyi, ji = i - ii * ncyi;
        Quad C;
        load_quad(xi, yi, nyi, ii, ji, C);
        const double orient = quad_area2(C) >= 0 ? 1.0 : -1.0;
        if (!convex(C, orient)) {
            atomicOr(flags, FLAG_NONCONVEX);
            continue;
        }
        // Sutherland-Hodgman: the output quad clipped by the 4 input edges
        PV poly[2][12];
        int m = 4;
        for (int v = 0; v < 4; v++) {
            PV& p = poly[0][v];
            p.x = O.x[v];
            p.y = O.y[v];
            p.ca = (signed char)((v + 3) & 3);
            p.cb = (signed char)v;
            p.kind = 0;
            p.e = (signed char)v;
            p.t = p.inv = 0;
        }
        int cur = 0;
        bool ok = true;
        for (int f = 0; f < 4 && m > 0; f++) {
            const double cx = C.x[f], cy = C.y[f];
            const double sx = C.x[(f + 1) & 3] - cx, sy = C.y[(f + 1) & 3] - cy;
            int n = 0;
            for (int v = 0; v < m; v++) {
                const PV& P = poly[cur][v];
                const PV& Q = poly[cur][(v + 1) % m];
                const bool pin = orient * cross2(sx, sy, P.x - cx, P.y - cy) >= 0;
                const bool qin = orient * cross2(sx, sy, Q.x - cx, Q.y - cy) >= 0;
                if (pin != qin && n < 12) poly[cur ^ 1][n++] = crossing(O, C, common_carrier(P, Q, &ok), f, &ok);
                if (qin && n < 12) poly[cur ^ 1][n++] = Q;
            }
            cur ^= 1;
            m = n;
        }
        if (!ok) atomicOr(flags, FLAG_DEGENERATE);
        if (m < 3) {
            if (w_check) w_check[k] = 0;
            continue;
        }
        const PV* p = poly[cur];
        double A2 = 0;
        for (int v = 0; v < m; v++) {
            const PV& a = p[v];
            const PV& b = p[(v + 1) % m];
            A2 += cross2(a.x, a.y, b.x, b.y);
        }
        const double ain = area_in[i];
        const double win = w_in ? w_in[i] : 1.0;
        double ratio = 0.5 * A2 / ain * win;
        // the stored weight fixes the sign convention (orientation of the grids)
        const double sgn = (val[k] * ratio < 0) ? -1.0 : 1.0;
        if (w_check) w_check[k] = sgn * ratio;
        if (G == 0) continue;
        const double c = G * sgn * win / ain;  // dL/dA
        for (int v = 0; v < m; v++) {
            const PV& q = p[v];
            if (q.kind == 1) continue;
            const PV& nx = p[(v + 1) % m];
            const PV& pv = p[(v + m - 1) % m];
            const double Gx = 0.5 * (nx.y - pv.y) * c, Gy = 0.5 * (pv.x - nx.x) * c;
            if (q.kind == 0) {
                ax[q.e] += Gx;
                ay[q.e] += Gy;
            } else {
                // the crossing of output edge e (r = b - a) with input edge f
                // (s): n = (-s.y, s.x) / cross(r, s)
                const int e0 = q.e, e1 = (q.e + 1) & 3, f0 = q.cb - 4, f1 = (q.cb - 3) & 3;
                const double rx = O.x[e1] - O.x[e0], ry = O.y[e1] - O.y[e0];
                const double nx = -(C.y[f1] - C.y[f0]) * q.inv, ny = (C.x[f1] - C.x[f0]) * q.inv;
                const double gr = Gx * rx + Gy * ry;
                const double hx = Gx + gr * nx, hy = Gy + gr * ny;
                const int a = q.e, b = (q.e + 1) & 3;
                ax[a] += (1 - q.t) * hx;
                ay[a] += (1 - q.t) * hy;
                ax[b] += q.t * hx;
                ay[b] += q.t * hy;
            }
        }
    }
    double* rec = corner + o * 8;
    for (int v = 0; v < 4; v++) {
        rec[v] = ax[v];
        rec[4 + v] = ay[v];
    }
}

// Gradient of output vertex (a, b): corner 0 of cell (a, b), corner 1 of
// cell (a - 1, b), corner 2 of cell (a - 1, b - 1) and corner 3 of cell
// (a, b - 1), those that exist, added in that order.
__global__ void __launch_bounds__(256)
    vertex_sum(const double* __restrict__ corner, int64_t nxo, int64_t nyo, double* __restrict__ gx,
               double* __restrict__ gy) {
    const int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= nxo * nyo) return;
    const int64_t a = v / nyo, b = v - a * nyo, ncy = nyo - 1;
    double sx = 0.0, sy = 0.0;
    const int64_t ci[4] = {a, a - 1, a - 1, a};
    const int64_t cj[4] = {b, b, b - 1, b - 1};
    for (int c = 0; c < 4; c++) {
        if (ci[c] < 0 || ci[c] >= nxo - 1 || cj[c] < 0 || cj[c] >= ncy) continue;
        const double* rec = corner + (ci[c] * ncy + cj[c]) * 8;
        sx += rec[c];
        sy += rec[4 + c];
    }
    gx[v] = sx;
    gy[v] = sy;
}

}  // namespace

int cell_area_2d(const double* x, const double* y, int64_t nx, int64_t ny, double* area, cudaStream_t s);

}  // namespace rg

extern "C" int rg_conservative_2d_grad_output(rg_weights w, const double* d_xi, const double* d_yi, int64_t nxi,
                                              int64_t nyi, const double* d_xo, const double* d_yo, int64_t nxo,
                                              int64_t nyo, const double* d_w_in, const void* d_values,
                                              const void* d_grad_out, int dtype, int64_t stack, double* d_grad_xo,
                                              double* d_grad_yo, double* d_w_check, rg_stream_t stream) {
    rg::NvtxRange nvtx_range("rg_conservative_2d_grad_output");
    using namespace rg;
    RG_CHECK(w, RG_ERR_ARG, "rg_conservative_2d_grad_output: NULL handle");
    RG_CHECK(nxi >= 2 && nyi >= 2 && nxo >= 2 && nyo >= 2, RG_ERR_ARG,
             "rg_conservative_2d_grad_output: grids need at least 2 vertices per axis");
    RG_CHECK(w->n_in == (nxi - 1) * (nyi - 1) && w->n_out == (nxo - 1) * (nyo - 1), RG_ERR_ARG,
             "rg_conservative_2d_grad_output: grids do not match the weights (%lld -> %lld cells)",
             (long long)w->n_in, (long long)w->n_out);
    RG_CHECK(dtype == RG_F32 || dtype == RG_F64, RG_ERR_ARG, "rg_conservative_2d_grad_output: bad dtype");
    RG_CHECK(stack >= 0, RG_ERR_ARG, "rg_conservative_2d_grad_output: negative stack");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t nv = nxo * nyo;
    if (w->n_out == 0 || w->nnz == 0) {
        RG_CUDA(cudaMemsetAsync(d_grad_xo, 0, sizeof(double) * nv, s));
        RG_CUDA(cudaMemsetAsync(d_grad_yo, 0, sizeof(double) * nv, s));
        return RG_OK;
    }
    double* area = nullptr;
    double* corner = nullptr;
    unsigned* flags = nullptr;
    int st = RG_OK;
    do {
        if ((st = dalloc(&area, (size_t)w->n_in, s))) break;
        if ((st = dalloc(&corner, (size_t)w->n_out * 8, s))) break;
        if ((st = dalloc(&flags, 1, s))) break;
        cudaMemsetAsync(flags, 0, sizeof(unsigned), s);
        if ((st = cell_area_2d(d_xi, d_yi, nxi, nyi, area, s))) break;
        const unsigned grid = grid_for(w->n_out, 128);
        if (dtype == RG_F32)
            grad_output_kernel<float><<<grid, 128, 0, s>>>(
                w->row_ptr, w->col, w->val, w->n_out, d_xi, d_yi, nyi, d_xo, d_yo, nyo, area, d_w_in,
                (const float*)d_values, (const float*)d_grad_out, w->n_in, stack, corner, d_w_check, flags);
        else
            grad_output_kernel<double><<<grid, 128, 0, s>>>(
                w->row_ptr, w->col, w->val, w->n_out, d_xi, d_yi, nyi, d_xo, d_yo, nyo, area, d_w_in,
                (const double*)d_values, (const double*)d_grad_out, w->n_in, stack, corner, d_w_check, flags);
        vertex_sum<<<grid_for(nv, 256), 256, 0, s>>>(corner, nxo, nyo, d_grad_xo, d_grad_yo);
        unsigned fl = 0;
        cudaMemcpyAsync(&fl, flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("rg_conservative_2d_grad_output: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }
        if (fl & FLAG_NONCONVEX) {
            set_error("rg_conservative_2d_grad_output: an input cell is not convex (the overlap clipping "
                      "needs convex input cells)");
            st = RG_ERR_UNSUPPORTED;
        } else if (fl & FLAG_DEGENERATE) {
            set_error("rg_conservative_2d_grad_output: degenerate overlap (parallel or coincident edges)");
            st = RG_ERR_UNSUPPORTED;
        }
    } while (0);
    dfree(area, s);
    dfree(corner, s);
    dfree(flags, s);
    return st;
}
