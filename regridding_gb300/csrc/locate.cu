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
// Points whose walk leaves the grid or exceeds its step cap are resolved by
// the winding number of the grid boundary (from y-binned boundary edges:
// zero means outside), and the rest by a lane-parallel exhaustive scan.  The
// allocation-free variant keeps the older fallback, a warp per point with a
// lane-parallel winding test over the whole boundary.
#include <cmath>
#include <mutex>

#include "common.cuh"
#include "seed.cuh"

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

__global__ void __launch_bounds__(128)
    locate_walk_kernel(G2 g, const double* __restrict__ px, const double* __restrict__ py, int64_t n,
                       int64_t* __restrict__ oi, int64_t* __restrict__ oj, int64_t* __restrict__ fails,
                       unsigned long long* __restrict__ nfail) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int64_t ncx = g.nx - 1, ncy = g.ny - 1;
    const double p_x = px[k], p_y = py[k];
    // starting guess: Newton on the bilinear index map (float32)
    int64_t ci, cj;
    seed_cell(g.x, g.y, g.nx, g.ny, p_x, p_y, &ci, &cj);
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

// ---------------------------------------------------------------------------
// Outside test with the grid boundary binned by y.  The extended winding
// number of a point sums a term over boundary edges, and only edges whose
// y-range contains the point's y give a non-zero term (a strict crossing or
// an endpoint at that y).  Edges are binned by y with the monotone map
// bin(v) = floor((v - ymin) * inv_h) (clamped), so an edge spanning
// [ylo, yhi] is filed in every bin from bin(ylo) to bin(yhi) and a point at y
// finds every edge it needs in bin(y).  The terms are +-1 and +-1/2, so their
// sum is exact in any order.  Bins whose fill would exceed the capacity set a
// flag and every point goes to the exhaustive scan instead.
// ---------------------------------------------------------------------------

struct YBins {
    double ymin, ymax, inv_h;
    int nbins;
};

__device__ __forceinline__ int ybin(const YBins& b, double v) {
    double f = floor(dmul(dsub(v, b.ymin), b.inv_h));
    if (!(f >= 0)) return 0;
    if (f >= (double)(b.nbins - 1)) return b.nbins - 1;
    return (int)f;
}

// one block: y-range of the boundary vertices -> bin parameters
__global__ void ybins_params(G2 g, int64_t nb, int nbins, YBins* out) {
    __shared__ double smin[256], smax[256];
    double lo = INFINITY, hi = -INFINITY;
    for (int64_t v = threadIdx.x; v < nb; v += blockDim.x) {
        double bx, by;
        bvertex(g, v, &bx, &by);
        lo = fmin(lo, by);
        hi = fmax(hi, by);
    }
    smin[threadIdx.x] = lo;
    smax[threadIdx.x] = hi;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + o]);
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        YBins b;
        b.ymin = smin[0];
        b.ymax = smax[0];
        b.nbins = nbins;
        double ext = dsub(b.ymax, b.ymin);
        b.inv_h = ext > 0 && isfinite(ext) ? ddiv((double)nbins, ext) : 0.0;
        *out = b;
    }
}

// PASS 0 counts the bins of every boundary edge; PASS 1 files the edges
template <int PASS>
__global__ void ybins_fill(G2 g, int64_t nb, const YBins* __restrict__ bp, unsigned* __restrict__ counts,
                           const int64_t* __restrict__ ptr, int32_t* __restrict__ items, int64_t cap,
                           unsigned* __restrict__ overflow) {
    const YBins b = *bp;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nb; e += (int64_t)gridDim.x * blockDim.x) {
        double ax, ay, bx, by;
        bvertex(g, e == 0 ? nb - 1 : e - 1, &ax, &ay);
        bvertex(g, e, &bx, &by);
        int b0 = ybin(b, fmin(ay, by)), b1 = ybin(b, fmax(ay, by));
        if (!(ay == ay) || !(by == by)) {  // NaN vertex: file it everywhere
            b0 = 0;
            b1 = b.nbins - 1;
        }
        for (int k = b0; k <= b1; k++) {
            unsigned pos = atomicAdd(&counts[k], 1u);
            if (PASS == 1) {
                int64_t at = ptr[k] + pos;
                if (at < cap) items[at] = (int32_t)e;
                else atomicOr(overflow, 1u);
            }
        }
    }
}

// thread per point the walk could not place: winding number from its bin;
// zero -> outside, otherwise the point goes to the exhaustive scan
__global__ void __launch_bounds__(128)
    locate_resolve_kernel(G2 g, int64_t nb, const double* __restrict__ px, const double* __restrict__ py,
                          const int64_t* __restrict__ fails, const unsigned long long* __restrict__ nfail,
                          const YBins* __restrict__ bp, const int64_t* __restrict__ ptr,
                          const int32_t* __restrict__ items, const int64_t* __restrict__ total,
                          const unsigned* __restrict__ overflow, int64_t cap, int64_t* __restrict__ hard,
                          unsigned long long* __restrict__ nhard, int64_t* __restrict__ oi,
                          int64_t* __restrict__ oj) {
    const unsigned long long nf = *nfail;
    const bool usable = *overflow == 0 && *total <= cap;
    const YBins b = *bp;
    for (unsigned long long w = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; w < nf;
         w += (unsigned long long)gridDim.x * blockDim.x) {
        const int64_t k = fails[w];
        const double x = px[k], y = py[k];
        bool inside = true;  // unknown: scan
        if (usable) {
            if (!(y >= b.ymin && y <= b.ymax)) {
                inside = false;
            } else {
                const int bin = ybin(b, y);
                double wn = 0;
                for (int64_t q = ptr[bin]; q < ptr[bin + 1]; q++) {
                    const int64_t e = items[q];
                    double ax, ay, bx, by;
                    bvertex(g, e == 0 ? nb - 1 : e - 1, &ax, &ay);
                    bvertex(g, e, &bx, &by);
                    wn += wterm(x, y, ax, ay, bx, by);
                }
                inside = wn != 0;
            }
        }
        if (inside) {
            hard[atomicAdd(nhard, 1ull)] = k;
        } else {
            oi[k] = MAXSIZE;
            oj[k] = MAXSIZE;
        }
    }
}

// warp per point inside the boundary that the walk missed: lowest-index
// containing cell by exhaustive scan (MAXSIZE if none)
__global__ void __launch_bounds__(128)
    locate_exhaustive_kernel(G2 g, const double* __restrict__ px, const double* __restrict__ py,
                             const int64_t* __restrict__ hard, const unsigned long long* __restrict__ nhard,
                             int64_t* __restrict__ oi, int64_t* __restrict__ oj) {
    const int lane = threadIdx.x & 31;
    const unsigned long long nh = *nhard;
    for (unsigned long long w = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5; w < nh;
         w += ((unsigned long long)gridDim.x * blockDim.x) >> 5) {
        const int64_t k = hard[w];
        const double x = px[k], y = py[k];
        int64_t ri = MAXSIZE, rj = MAXSIZE;
        const int64_t ncy = g.ny - 1, ncells = (g.nx - 1) * ncy;
        for (int64_t base = 0; base < ncells; base += 32) {
            const int64_t c = base + lane;
            const bool hit = c < ncells && contains(g, c / ncy, c % ncy, x, y);
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (m) {
                const int64_t cc = base + __ffs(m) - 1;
                ri = cc / ncy;
                rj = cc % ncy;
                break;
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
    const int64_t nb = 2 * (nx - 1) + 2 * (ny - 1);
    int64_t nbins64 = nb / 2;
    if (nbins64 < 1) nbins64 = 1;
    if (nbins64 > (1 << 16)) nbins64 = 1 << 16;
    const int nbins = (int)nbins64;
    const int64_t cap = 8 * nb + 2 * nbins64;
    int64_t *fails = nullptr, *hard = nullptr, *ptr = nullptr, *total = nullptr;
    unsigned long long* nfail = nullptr;  // [0] walk failures, [1] points for the exhaustive scan
    unsigned *counts = nullptr, *overflow = nullptr;
    int32_t* items = nullptr;
    YBins* bp = nullptr;
    int st = RG_OK;
    do {
        if ((st = dalloc(&fails, (size_t)n, s))) break;
        if ((st = dalloc(&hard, (size_t)n, s))) break;
        if ((st = dalloc(&nfail, 2, s))) break;
        if ((st = dalloc(&counts, (size_t)nbins + 1, s))) break;
        if ((st = dalloc(&overflow, 1, s))) break;
        if ((st = dalloc(&ptr, (size_t)nbins + 1, s))) break;
        if ((st = dalloc(&total, 1, s))) break;
        if ((st = dalloc(&items, (size_t)cap, s))) break;
        if ((st = dalloc(&bp, 1, s))) break;
        cudaMemsetAsync(nfail, 0, 2 * sizeof(unsigned long long), s);
        cudaMemsetAsync(counts, 0, sizeof(unsigned) * (nbins + 1), s);
        cudaMemsetAsync(overflow, 0, sizeof(unsigned), s);
        G2 g{x, y, nx, ny};
        const unsigned eb = grid_for(nb, 128) > 1024 ? 1024 : grid_for(nb, 128);
        ybins_params<<<1, 256, 0, s>>>(g, nb, nbins, bp);
        ybins_fill<0><<<eb, 128, 0, s>>>(g, nb, bp, counts, nullptr, nullptr, cap, overflow);
        if ((st = exclusive_scan_u32_to_i64(counts, ptr, nbins + 1, total, s))) break;
        cudaMemsetAsync(counts, 0, sizeof(unsigned) * (nbins + 1), s);
        ybins_fill<1><<<eb, 128, 0, s>>>(g, nb, bp, counts, ptr, items, cap, overflow);
        locate_walk_kernel<<<grid_for(n, 128), 128, 0, s>>>(g, px, py, n, oi, oj, fails, nfail);
        locate_resolve_kernel<<<1024, 128, 0, s>>>(g, nb, px, py, fails, nfail, bp, ptr, items, total, overflow,
                                                   cap, hard, nfail + 1, oi, oj);
        locate_exhaustive_kernel<<<1024, 128, 0, s>>>(g, px, py, hard, nfail + 1, oi, oj);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error("locate_2d_walk: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
        }
    } while (0);
    dfree(fails, s);
    dfree(hard, s);
    dfree(nfail, s);
    dfree(counts, s);
    dfree(overflow, s);
    dfree(ptr, s);
    dfree(total, s);
    dfree(items, s);
    dfree(bp, s);
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
// once per device, with that device current, and kept until the process
// exits (a device reset after the first call is not supported).
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
