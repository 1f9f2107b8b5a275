// Fast point location in a curvilinear 2D grid (new public 2D find_indices).
//
// The exhaustive upstream locator (index_of_point_brute,
// regridding/_weights/_weights_conservative_2d/_grids.py:218-279) returns the
// lowest-index cell whose quad contains the point.  Here each thread seeds a
// guess with a few Newton steps on the bilinear index map, then walks from
// cell to cell across the edge the point lies beyond until the exact
// containment test (the extended winding number of geometry.py:737-829)
// succeeds, and finally takes the lowest-index containing cell among the 3x3
// neighbourhood, which is the exhaustive answer whenever cells do not overlap.
// Points whose walk leaves the grid or exceeds its step cap are resolved by a
// warp each: a lane-parallel winding test against the whole grid boundary
// decides "outside", otherwise a lane-parallel exhaustive scan answers.
#include <cmath>
#include <mutex>

#include "common.cuh"

namespace rg {
namespace {

struct G2 {
    const double* x;
    const double* y;
    int64_t nx, ny;
    __device__ __forceinline__ double X(int64_t i, int64_t j) const { return __ldg(x + i * ny + j); }
    __device__ __forceinline__ double Y(int64_t i, int64_t j) const { return __ldg(y + i * ny + j); }
};

__device__ __forceinline__ double wterm(double x, double y, double vx0, double vy0, double vx1,
                                        double vy1) {
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

__device__ bool contains(const G2& g, int64_t i, int64_t j, double px, double py) {
    double vx[4] = {g.X(i, j), g.X(i + 1, j), g.X(i + 1, j + 1), g.X(i, j + 1)};
    double vy[4] = {g.Y(i, j), g.Y(i + 1, j), g.Y(i + 1, j + 1), g.Y(i, j + 1)};
    double w = 0;
#pragma unroll
    for (int v = 0; v < 4; v++) {
        int p = (v + 3) & 3;
        w = w + wterm(px, py, vx[p], vy[p], vx[v], vy[v]);
    }
    return w != 0;
}

__device__ void lowest_local(const G2& g, double px, double py, int64_t i0, int64_t j0, int64_t* oi,
                             int64_t* oj) {
    int64_t ncx = g.nx - 1, ncy = g.ny - 1;
    int64_t ia = i0 - 1 > 0 ? i0 - 1 : 0, ib = i0 + 2 < ncx ? i0 + 2 : ncx;
    int64_t ja = j0 - 1 > 0 ? j0 - 1 : 0, jb = j0 + 2 < ncy ? j0 + 2 : ncy;
    for (int64_t ii = ia; ii < ib; ii++)
        for (int64_t jj = ja; jj < jb; jj++)
            if (contains(g, ii, jj, px, py)) {
                *oi = ii;
                *oj = jj;
                return;
            }
    *oi = i0;
    *oj = j0;
}

__device__ __forceinline__ double bilin(const double* a, int64_t sx, int64_t sy, double x, double y) {
    int64_t x0 = (int64_t)floor(x), y0 = (int64_t)floor(y);
    x0 = x0 < 0 ? 0 : (x0 > sx - 2 ? sx - 2 : x0);
    y0 = y0 < 0 ? 0 : (y0 > sy - 2 ? sy - 2 : y0);
    double dx = x - x0, dy = y - y0;
    double a00 = __ldg(a + x0 * sy + y0), a01 = __ldg(a + x0 * sy + y0 + 1);
    double a10 = __ldg(a + (x0 + 1) * sy + y0), a11 = __ldg(a + (x0 + 1) * sy + y0 + 1);
    return a00 * (1 - dx) * (1 - dy) + a01 * (1 - dx) * dy + a10 * dx * (1 - dy) + a11 * dx * dy;
}

__global__ void __launch_bounds__(128)
    locate_walk_kernel(G2 g, const double* __restrict__ px, const double* __restrict__ py, int64_t n,
                       int64_t* __restrict__ oi, int64_t* __restrict__ oj, int64_t* __restrict__ fails,
                       unsigned long long* __restrict__ nfail) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int64_t ncx = g.nx - 1, ncy = g.ny - 1;
    const double p_x = px[k], p_y = py[k];
    // Newton seed on the bilinear index map (forward differences)
    double fi = 0.5 * (double)ncx, fj = 0.5 * (double)ncy;
    for (int it = 0; it < 12; it++) {
        double xv = bilin(g.x, g.nx, g.ny, fi, fj), yv = bilin(g.y, g.nx, g.ny, fi, fj);
        double ex = xv - p_x, ey = yv - p_y;
        const double h = 1e-3;
        double xi = (bilin(g.x, g.nx, g.ny, fi + h, fj) - xv) / h;
        double xj = (bilin(g.x, g.nx, g.ny, fi, fj + h) - xv) / h;
        double yi = (bilin(g.y, g.nx, g.ny, fi + h, fj) - yv) / h;
        double yj = (bilin(g.y, g.nx, g.ny, fi, fj + h) - yv) / h;
        double det = xi * yj - xj * yi;
        if (!(det != 0) || !isfinite(det)) break;
        double di = (yj * ex - xj * ey) / det, dj = (-yi * ex + xi * ey) / det;
        fi -= di;
        fj -= dj;
        fi = fmin(fmax(fi, 0.0), (double)ncx - 1e-9);
        fj = fmin(fmax(fj, 0.0), (double)ncy - 1e-9);
        if (fabs(di) < 1e-3 && fabs(dj) < 1e-3) break;
    }
    int64_t ci = (int64_t)floor(fi), cj = (int64_t)floor(fj);
    ci = ci < 0 ? 0 : (ci >= ncx ? ncx - 1 : ci);
    cj = cj < 0 ? 0 : (cj >= ncy ? ncy - 1 : cj);
    const int cap = 64 + 2 * (int)sqrt((double)(ncx + ncy));
    for (int step = 0; step < cap; step++) {
        if (contains(g, ci, cj, p_x, p_y)) {
            int64_t ri, rj;
            lowest_local(g, p_x, p_y, ci, cj, &ri, &rj);
            oi[k] = ri;
            oj[k] = rj;
            return;
        }
        // cross the edge the point lies furthest beyond (orientation aware)
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
            double cr = sgn * (ex * (p_y - vy[e]) - ey * (p_x - vx[e]));
            double len = sqrt(ex * ex + ey * ey);
            double sc = len > 0 ? cr / len : 0;
            if (sc < worst) {
                worst = sc;
                best = e;
            }
        }
        if (best < 0) break;  // numerically inside every edge yet not contained: give up
        // edge e of the cell (v_e -> v_e+1) borders: 0 -> (i, j-1), 1 -> (i+1, j), 2 -> (i, j+1), 3 -> (i-1, j)
        const int di[4] = {0, 1, 0, -1};
        const int dj[4] = {-1, 0, 1, 0};
        int64_t ni = ci + di[best], nj = cj + dj[best];
        if (ni < 0 || nj < 0 || ni >= ncx || nj >= ncy) break;
        ci = ni;
        cj = nj;
    }
    unsigned long long slot = atomicAdd(nfail, 1ull);
    fails[slot] = k;
}

__device__ __forceinline__ void bvertex(const G2& g, int64_t k, double* bx, double* by) {
    int64_t sx = g.nx, sy = g.ny, i, j;
    if (k < sx - 1) { i = k; j = 0; }
    else if ((k -= sx - 1) < sy - 1) { i = sx - 1; j = k; }
    else if ((k -= sy - 1) < sx - 1) { i = sx - 1 - k; j = sy - 1; }
    else { k -= sx - 1; i = 0; j = sy - 1 - k; }
    *bx = g.X(i, j);
    *by = g.Y(i, j);
}

// warp per unresolved point
__global__ void __launch_bounds__(128)
    locate_fallback_kernel(G2 g, const double* __restrict__ px, const double* __restrict__ py,
                           const int64_t* __restrict__ fails, const unsigned long long* __restrict__ nfail,
                           int64_t* __restrict__ oi, int64_t* __restrict__ oj) {
    int lane = threadIdx.x & 31;
    unsigned long long nf = *nfail;
    for (unsigned long long w = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5; w < nf;
         w += ((unsigned long long)gridDim.x * blockDim.x) >> 5) {
        int64_t k = fails[w];
        double x = px[k], y = py[k];
        int64_t nb = 2 * (g.nx - 1) + 2 * (g.ny - 1);
        double wn = 0;
        for (int64_t v = lane; v < nb; v += 32) {
            double ax, ay, bx, by;
            bvertex(g, v == 0 ? nb - 1 : v - 1, &ax, &ay);
            bvertex(g, v, &bx, &by);
            wn += wterm(x, y, ax, ay, bx, by);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) wn += __shfl_xor_sync(0xffffffffu, wn, o);
        int64_t ri = MAXSIZE, rj = MAXSIZE;
        if (wn != 0) {
            int64_t ncy = g.ny - 1, ncells = (g.nx - 1) * ncy;
            for (int64_t base = 0; base < ncells; base += 32) {
                int64_t c = base + lane;
                bool hit = c < ncells && contains(g, c / ncy, c % ncy, x, y);
                unsigned m = __ballot_sync(0xffffffffu, hit);
                if (m) {
                    int64_t cc = base + __ffs(m) - 1;
                    ri = cc / ncy;
                    rj = cc % ncy;
                    break;
                }
            }
        }
        if (lane == 0) {
            oi[k] = ri;
            oj[k] = rj;
        }
    }
}

}  // namespace

int locate_2d_walk(const double* x, const double* y, int64_t nx, int64_t ny, const double* px,
                   const double* py, int64_t n, int64_t* oi, int64_t* oj, cudaStream_t s) {
    if (n <= 0) return RG_OK;
    int64_t* fails = nullptr;
    unsigned long long* nfail = nullptr;
    RG_TRY(dalloc(&fails, (size_t)n, s));
    int st = dalloc(&nfail, 1, s);
    if (st == RG_OK) {
        cudaMemsetAsync(nfail, 0, sizeof(unsigned long long), s);
        G2 g{x, y, nx, ny};
        locate_walk_kernel<<<grid_for(n, 128), 128, 0, s>>>(g, px, py, n, oi, oj, fails, nfail);
        locate_fallback_kernel<<<1024, 128, 0, s>>>(g, px, py, fails, nfail, oi, oj);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error("locate_2d_walk: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
        }
    }
    dfree(fails, s);
    dfree(nfail, s);
    return st;
}

}  // namespace rg

// ---------------------------------------------------------------------------
// Allocation-free variant of the walk locator.
//
// Some callers cannot allocate device memory at call time: a host process
// whose device memory is entirely owned by another allocator (a framework
// pool or a fixed serving budget), or a latency-critical loop that must not
// risk the implicit synchronisation or the out-of-memory failure of an
// allocation in the middle of its work.  For them, the only scratch the
// walk locator needs -- the list of points the walk hands to the warp
// fallback, and its counter -- lives in the file-scope array below, which
// the CUDA runtime places in device memory once per device when the library
// is loaded there and keeps until the process exits.
// ---------------------------------------------------------------------------
namespace rg {
namespace {

constexpr int64_t kNoallocMaxPoints = RG_LOCATE_NOALLOC_MAX_POINTS;

// word 0: number of points left to the fallback; words 32..: their indices
static __device__ __align__(256) unsigned long long g_locate_scratch[32 + kNoallocMaxPoints];

std::mutex g_scratch_mutex;
void* g_scratch_address[256] = {};  // per device ordinal, filled on first use

// Device address of g_locate_scratch on the current device.  In host code the
// array's name only stands in for the symbol, so the address is looked up
// once per device, with that device current.
int scratch_address(void** out) {
    int dev = 0;
    RG_CUDA(cudaGetDevice(&dev));
    RG_CHECK(dev >= 0 && dev < 256, RG_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_address[dev] == nullptr) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_locate_scratch);
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_error("rg_locate_2d_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return RG_ERR_CUDA;
        }
        g_scratch_address[dev] = p;
    }
    *out = g_scratch_address[dev];
    return RG_OK;
}

}  // namespace
}  // namespace rg

extern "C" int rg_locate_2d_noalloc(const double* d_x, const double* d_y, int64_t nx, int64_t ny,
                                    const double* d_px, const double* d_py, int64_t npts, int64_t* d_i,
                                    int64_t* d_j, rg_stream_t stream) {
    using namespace rg;
    RG_CHECK(nx >= 2 && ny >= 2, RG_ERR_ARG, "rg_locate_2d_noalloc: need at least 2x2 vertices");
    RG_CHECK(npts >= 0 && npts <= kNoallocMaxPoints, RG_ERR_ARG,
             "rg_locate_2d_noalloc: %lld points requested, at most %lld per call (split the call, or use "
             "rg_locate_2d, which allocates its scratch)",
             (long long)npts, (long long)kNoallocMaxPoints);
    if (npts == 0) return RG_OK;
    void* base = nullptr;
    RG_TRY(scratch_address(&base));
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long* nfail = (unsigned long long*)base;
    int64_t* fails = (int64_t*)((unsigned long long*)base + 32);
    // the array keeps the previous call's contents: the counter starts at zero
    RG_CUDA(cudaMemsetAsync(nfail, 0, sizeof(unsigned long long), s));
    G2 g{d_x, d_y, nx, ny};
    locate_walk_kernel<<<grid_for(npts, 128), 128, 0, s>>>(g, d_px, d_py, npts, d_i, d_j, fails, nfail);
    locate_fallback_kernel<<<1024, 128, 0, s>>>(g, d_px, d_py, fails, nfail, d_i, d_j);
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}
