// fill(method="gauss_seidel"): red-black Gauss-Seidel relaxation of the
// missing cells of a stack of 2D slices (regridding/_fill/_gauss_seidel.py
// :12-139), and the per-slice median of the valid cells that seeds it
// (_guess_median, :61-80).
//
// Layout: a stack of nt slices of ny x nx cells, C-ordered, float64 or
// float32, and a byte mask `where` of the same shape (1 = missing).
//
// Relaxation.  The upstream visits, for every slice, iteration and colour
// (even cells (i + j) & 1 == 0 first, then odd), the cells of that colour in
// row-major order and replaces each missing one with
//     (dxxinv * (a[j, i-1] + a[j, i+1]) + dyyinv * (a[j-1, i] + a[j+1, i])) * dcent
// with periodic neighbours.  Cells of one colour only read cells of the other
// colour, except across the periodic seam of an odd axis: with nx odd, column
// nx - 1 has the colour of column 0 in every row, so (j, 0) reads the old
// (j, nx - 1) and (j, nx - 1) then reads the new (j, 0); likewise rows 0 and
// ny - 1 for ny odd.  Each colour is therefore split into three phases run in
// order: cells off the odd seams, cells on exactly one seam (last column or
// last row), and the last corner.  Cells within a phase never read one
// another, so one launch updates a phase of every slice at once and the
// result equals the sequential sweep bit for bit.  The missing cells of each
// (colour, phase) class are compacted once, in (slice, cell) order, into a
// list of 64-bit entries (slice << 32 | cell); every iteration is then six
// gather launches over the lists, and cells that are not missing cost
// nothing.  Per updated cell: 6 FP64 operations, 4 neighbour reads, 1 write.
//
// Median.  A radix select on order-preserving integer keys of the valid,
// non-NaN values (8-bit digits, most significant first: 8 histogram passes
// for float64, 4 for float32), then one pass for the element following the
// lower median; the median is (lo + hi) / 2 in the array's dtype for an even
// count (numpy's mean of the two middle elements), the middle element for an
// odd count, and 0 for a slice without valid values.
#include "common.cuh"

namespace rg {
namespace {

constexpr int kClasses = 6;  // colour (2) x phase (3)
constexpr int kClassifyThreads = 256;
constexpr int kClassifyItems = 16;
constexpr int64_t kTile = (int64_t)kClassifyThreads * kClassifyItems;

__device__ __forceinline__ int cell_class(uint32_t j, uint32_t i, uint32_t ny, uint32_t nx) {
    const int colour = (int)((i + j) & 1u);
    const int phase = (int)((nx & 1u) && i == nx - 1) + (int)((ny & 1u) && j == ny - 1);
    return colour * 3 + phase;
}

// class of cell c of slice t, or -1 when it is not missing / past the slice
__device__ __forceinline__ int missing_class(const uint8_t* __restrict__ where, uint64_t slice_base, uint32_t c,
                                             uint32_t S, uint32_t ny, uint32_t nx) {
    if (c >= S || !where[slice_base + c]) return -1;
    const uint32_t j = c / nx;
    return cell_class(j, c - j * nx, ny, nx);
}

// Pass 1: missing cells per (class, tile); counts laid out [class][block]
// with block = t * tiles + tile.
__global__ void __launch_bounds__(kClassifyThreads) fill_count(const uint8_t* __restrict__ where, int64_t nt,
                                                               uint32_t ny, uint32_t nx, int64_t tiles,
                                                               unsigned* __restrict__ counts) {
    __shared__ unsigned sc[kClasses];
    const uint32_t S = ny * nx;
    const int64_t nblocks = nt * tiles;
    for (int64_t t = blockIdx.y; t < nt; t += gridDim.y) {
        if (threadIdx.x < kClasses) sc[threadIdx.x] = 0;
        __syncthreads();
        unsigned local[kClasses] = {0, 0, 0, 0, 0, 0};
        const uint64_t base = (uint64_t)t * S;
        const uint32_t c0 = (uint32_t)(blockIdx.x * kTile);
        for (int r = 0; r < kClassifyItems; ++r) {
            const int cls = missing_class(where, base, c0 + r * kClassifyThreads + threadIdx.x, S, ny, nx);
#pragma unroll
            for (int k = 0; k < kClasses; ++k) local[k] += cls == k;
        }
#pragma unroll
        for (int k = 0; k < kClasses; ++k)
            if (local[k]) atomicAdd(&sc[k], local[k]);
        __syncthreads();
        if (threadIdx.x < kClasses) counts[threadIdx.x * nblocks + t * tiles + blockIdx.x] = sc[threadIdx.x];
        __syncthreads();
    }
}

// Pass 2: write the entries of every class in (slice, cell) order: warp
// ballots give each missing cell its rank among the tile's cells of its
// class, on top of the scanned offset of (class, block).
__global__ void __launch_bounds__(kClassifyThreads) fill_lists(const uint8_t* __restrict__ where, int64_t nt,
                                                               uint32_t ny, uint32_t nx, int64_t tiles,
                                                               const int64_t* __restrict__ offsets,
                                                               uint64_t* __restrict__ list) {
    constexpr int kWarps = kClassifyThreads / 32;
    __shared__ unsigned wc[kWarps][kClasses];
    __shared__ int64_t run[kClasses];
    const uint32_t S = ny * nx;
    const int64_t nblocks = nt * tiles;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    for (int64_t t = blockIdx.y; t < nt; t += gridDim.y) {
        if (threadIdx.x < kClasses) run[threadIdx.x] = offsets[threadIdx.x * nblocks + t * tiles + blockIdx.x];
        const uint64_t base = (uint64_t)t * S;
        const uint32_t c0 = (uint32_t)(blockIdx.x * kTile);
        for (int r = 0; r < kClassifyItems; ++r) {
            const uint32_t c = c0 + r * kClassifyThreads + threadIdx.x;
            const int cls = missing_class(where, base, c, S, ny, nx);
            unsigned mine = 0;
#pragma unroll
            for (int k = 0; k < kClasses; ++k) {
                const unsigned b = __ballot_sync(0xffffffffu, cls == k);
                if (lane == 0) wc[warp][k] = __popc(b);
                if (cls == k) mine = __popc(b & lt);
            }
            __syncthreads();
            if (cls >= 0) {
                int64_t pos = run[cls] + mine;
                for (int w = 0; w < warp; ++w) pos += wc[w][cls];
                list[pos] = ((uint64_t)t << 32) | c;
            }
            __syncthreads();
            if (threadIdx.x < kClasses) {
                unsigned tot = 0;
                for (int w = 0; w < kWarps; ++w) tot += wc[w][threadIdx.x];
                run[threadIdx.x] += tot;
            }
            __syncthreads();
        }
    }
}

// the start of every class in the scanned offsets, and the total
__global__ void fill_class_starts(const int64_t* __restrict__ offsets, int64_t nblocks, int64_t* __restrict__ out) {
    const int k = threadIdx.x;
    if (k <= kClasses) out[k] = offsets[k * nblocks];
}

struct GsConst {
    double dxxinv, dyyinv, dcent;
};

// _iteration_gauss_seidel_2d (:110-139), float64: every operation rounds once.
__device__ __forceinline__ double gs_value(double l, double r, double d, double u, const GsConst& k) {
    return dmul(dadd(dmul(k.dxxinv, dadd(l, r)), dmul(k.dyyinv, dadd(d, u))), k.dcent);
}
// float32 arrays under Numba's typing: float32 neighbour sums, float64
// products and sum, the result rounded to float32 on store.
__device__ __forceinline__ float gs_value(float l, float r, float d, float u, const GsConst& k) {
    const double xs = (double)__fadd_rn(l, r), ys = (double)__fadd_rn(d, u);
    return __double2float_rn(dmul(dadd(dmul(k.dxxinv, xs), dmul(k.dyyinv, ys)), k.dcent));
}

// kFillEntries list entries per thread, all their neighbour loads issued
// before any store: cells of one class never read one another, so the order
// is free, and the extra loads in flight hide the gather latency.
constexpr int kFillEntries = 2;  // 4 measured slower (86 against 82 us per iteration)

template <typename T>
__global__ void fill_update(T* __restrict__ a, const uint64_t* __restrict__ list, int64_t n, uint32_t ny,
                            FastDiv nx_div, GsConst k) {
    const uint32_t nx = nx_div.d;
    const uint64_t S = (uint64_t)ny * nx;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += kFillEntries * stride) {
        T v[kFillEntries][4];
        T* dst[kFillEntries];
#pragma unroll
        for (int h = 0; h < kFillEntries; ++h) dst[h] = nullptr;
#pragma unroll
        for (int h = 0; h < kFillEntries; ++h) {
            const int64_t qq = q + h * stride;
            if (qq >= n) break;
            const uint64_t e = list[qq];
            const uint32_t c = (uint32_t)e;
            T* s = a + (e >> 32) * S;
            const uint32_t j = nx_div.div(c), i = c - j * nx;
            const uint32_t i9 = i ? i - 1 : nx - 1, i1 = i + 1 == nx ? 0 : i + 1;
            const uint32_t j9 = j ? j - 1 : ny - 1, j1 = j + 1 == ny ? 0 : j + 1;
            const T* row = s + (uint64_t)j * nx;
            v[h][0] = row[i9];
            v[h][1] = row[i1];
            v[h][2] = s[(uint64_t)j9 * nx + i];
            v[h][3] = s[(uint64_t)j1 * nx + i];
            dst[h] = s + c;
        }
#pragma unroll
        for (int h = 0; h < kFillEntries; ++h)
            if (dst[h]) *dst[h] = gs_value(v[h][0], v[h][1], v[h][2], v[h][3], k);
    }
}

// a[where] = guess: one value per slice (kind 1) or one per cell (kind 2)
template <typename T>
__global__ void fill_seed(T* __restrict__ a, const uint8_t* __restrict__ where, int64_t nt, int64_t S,
                          const T* __restrict__ guess, int full) {
    for (int64_t t = blockIdx.y; t < nt; t += gridDim.y) {
        for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < S; c += (int64_t)gridDim.x * blockDim.x) {
            const int64_t idx = t * S + c;
            if (where[idx]) a[idx] = full ? guess[idx] : guess[t];
        }
    }
}

// ---------------------------------------------------------------------------
// per-slice median
// ---------------------------------------------------------------------------

template <typename T>
struct Keys;
template <>
struct Keys<double> {
    using K = unsigned long long;
    static constexpr int kBits = 64;
    __device__ static K key(double v) {
        const K u = (K)__double_as_longlong(v);
        return (u >> 63) ? ~u : (u | (1ull << 63));
    }
    __device__ static double value(K k) {
        const K u = (k >> 63) ? (k & ~(1ull << 63)) : ~k;
        return __longlong_as_double((long long)u);
    }
    __device__ static double mid(double lo, double hi) { return dmul(dadd(lo, hi), 0.5); }
    // NaN test on the bits: keeps the FP64 pipe (2 lanes per clock per SM) out of the scans
    __device__ static bool is_nan(double v) {
        return ((unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
    }
};
template <>
struct Keys<float> {
    using K = unsigned;
    static constexpr int kBits = 32;
    __device__ static K key(float v) {
        const K u = (K)__float_as_uint(v);
        return (u >> 31) ? ~u : (u | (1u << 31));
    }
    __device__ static float value(K k) {
        const K u = (k >> 31) ? (k & ~(1u << 31)) : ~k;
        return __uint_as_float(u);
    }
    __device__ static float mid(float lo, float hi) { return __fmul_rn(__fadd_rn(lo, hi), 0.5f); }
    __device__ static bool is_nan(float v) { return (__float_as_uint(v) & 0x7fffffffu) > 0x7f800000u; }
};

struct MedianState {
    unsigned long long prefix, mask;  // digits of the lower median's key chosen so far
    unsigned long long min_above;     // smallest valid key above the candidate range
    unsigned long long min_gt;        // smallest candidate key above the lower median
    unsigned long long count_le;      // candidate keys <= the lower median
    long long n, k;                   // valid count, rank still to find within the prefix
    long long below;                  // valid keys below the candidate range
    long long cand;                   // valid keys within it (the candidates)
};

// The two leading digits are chosen from histograms over the whole stack;
// the keys that share them (a small fraction of real data) are then copied
// out and the remaining digits are chosen from histograms of those copies.
constexpr int kDataPasses = 2;

// Values read per thread before they are used, so that enough loads are in
// flight to stream the stack at HBM speed.
constexpr int kMedianUnroll = 8;

// add `bin` (0xffffffff: nothing) to the block histogram; the lanes of a
// warp that share a bin add to it once (the leading digits of real data fall
// into a few bins, where per-lane atomics would serialise)
__device__ __forceinline__ void hist_add(unsigned* h, unsigned bin, unsigned lane) {
    if (!__any_sync(0xffffffffu, bin != 0xffffffffu)) return;
    const unsigned peers = __match_any_sync(0xffffffffu, bin);
    if (bin != 0xffffffffu && (unsigned)(__ffs(peers) - 1) == lane) atomicAdd(&h[bin], __popc(peers));
}

// histogram of the next digit over the valid keys of the stack that match
// the prefix
template <typename T>
__global__ void median_hist(const T* __restrict__ a, const uint8_t* __restrict__ where, int64_t nt, int64_t S,
                            int shift, const MedianState* __restrict__ st, unsigned* __restrict__ hist) {
    using KT = Keys<T>;
    __shared__ unsigned h[256];
    const unsigned lane = threadIdx.x & 31u;
    const int64_t span = (int64_t)blockDim.x * kMedianUnroll;
    for (int64_t t = blockIdx.y; t < nt; t += gridDim.y) {
        for (int b = threadIdx.x; b < 256; b += blockDim.x) h[b] = 0;
        __syncthreads();
        const unsigned long long prefix = st[t].prefix, mask = st[t].mask;
        const T* s = a + t * S;
        const uint8_t* w = where + t * S;
        // the trip count is uniform over the block, so whole warps take part
        for (int64_t base = blockIdx.x * span; base < S; base += (int64_t)gridDim.x * span) {
            T v[kMedianUnroll];
            bool ok[kMedianUnroll];
#pragma unroll
            for (int u = 0; u < kMedianUnroll; ++u) {
                const int64_t c = base + u * (int64_t)blockDim.x + threadIdx.x;
                ok[u] = c < S;
                if (ok[u]) {
                    v[u] = s[c];
                    ok[u] = !w[c];
                }
            }
#pragma unroll
            for (int u = 0; u < kMedianUnroll; ++u) {
                unsigned bin = 0xffffffffu;
                if (ok[u] && !KT::is_nan(v[u])) {
                    const unsigned long long key = KT::key(v[u]);
                    if ((key & mask) == prefix) bin = (unsigned)(key >> shift) & 255u;
                }
                hist_add(h, bin, lane);
            }
        }
        __syncthreads();
        for (int b = threadIdx.x; b < 256; b += blockDim.x)
            if (h[b]) atomicAdd(&hist[t * 256 + b], h[b]);
        __syncthreads();
    }
}

// the same over the copied candidate keys of each slice
__global__ void median_hist_keys(const unsigned long long* __restrict__ keys, const int64_t* __restrict__ offsets,
                                 int64_t nt, int shift, const MedianState* __restrict__ st,
                                 unsigned* __restrict__ hist) {
    __shared__ unsigned h[256];
    const unsigned lane = threadIdx.x & 31u;
    for (int64_t t = blockIdx.y; t < nt; t += gridDim.y) {
        for (int b = threadIdx.x; b < 256; b += blockDim.x) h[b] = 0;
        __syncthreads();
        const unsigned long long prefix = st[t].prefix, mask = st[t].mask;
        const int64_t lo = offsets[t], hi = offsets[t + 1];
        for (int64_t base = lo + blockIdx.x * (int64_t)blockDim.x; base < hi; base += (int64_t)gridDim.x * blockDim.x) {
            const int64_t c = base + threadIdx.x;
            unsigned bin = 0xffffffffu;
            if (c < hi) {
                const unsigned long long key = keys[c];
                if ((key & mask) == prefix) bin = (unsigned)(key >> shift) & 255u;
            }
            hist_add(h, bin, lane);
        }
        __syncthreads();
        for (int b = threadIdx.x; b < 256; b += blockDim.x)
            if (h[b]) atomicAdd(&hist[t * 256 + b], h[b]);
        __syncthreads();
    }
}

// One warp per slice chooses the digit holding rank k (the first pass
// counts the valid keys, which fixes k) and clears the histogram.
__global__ void median_pick(MedianState* __restrict__ st, unsigned* __restrict__ hist, int64_t nt, int shift,
                            int pass) {
    const int64_t t = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31u;
    if (t >= nt) return;  // whole warps
    unsigned* h = hist + t * 256 + lane * 8;
    unsigned c[8];
    long long mine = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        c[q] = h[q];
        mine += c[q];
        h[q] = 0;
    }
    long long incl = mine;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const long long up = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= (unsigned)d) incl += up;
    }
    const long long total = __shfl_sync(0xffffffffu, incl, 31);
    MedianState s = st[t];
    if (pass == 0) {
        s.n = total;
        s.k = total > 0 ? (total - 1) / 2 : 0;
    }
    if (s.n == 0) {
        if (lane == 0 && pass == 0) st[t] = s;
        return;
    }
    const long long excl = incl - mine;
    const unsigned owner = __ffs(__ballot_sync(0xffffffffu, excl <= s.k && s.k < incl)) - 1;
    if (lane != owner) return;
    long long acc = excl;
    int q = 0;
    for (; q < 7; ++q) {
        if (acc + (long long)c[q] > s.k) break;
        acc += c[q];
    }
    const int b = (int)lane * 8 + q;
    s.k -= acc;
    if (pass < kDataPasses) s.below += acc;
    s.cand = c[q];
    s.prefix |= (unsigned long long)b << shift;
    s.mask |= 255ull << shift;
    st[t] = s;
}

__global__ void median_cand_counts(const MedianState* __restrict__ st, int64_t nt, int64_t* __restrict__ counts) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < nt) counts[t] = st[t].n > 0 ? st[t].cand : 0;
    if (t == nt) counts[t] = 0;
}

// copy the valid keys within the candidate range (warp-aggregated slots)
// and find the smallest valid key above it
template <typename T>
__global__ void median_compact(const T* __restrict__ a, const uint8_t* __restrict__ where, int64_t nt, int64_t S,
                               MedianState* __restrict__ st, const int64_t* __restrict__ offsets,
                               unsigned long long* __restrict__ cursor, unsigned long long* __restrict__ keys) {
    using KT = Keys<T>;
    __shared__ unsigned long long above;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t span = (int64_t)blockDim.x * kMedianUnroll;
    for (int64_t t = blockIdx.y; t < nt; t += gridDim.y) {
        if (threadIdx.x == 0) above = ~0ull;
        __syncthreads();
        const unsigned long long prefix = st[t].prefix, mask = st[t].mask;
        const bool any = st[t].n > 0;
        const int64_t out0 = offsets[t];
        unsigned long long my_above = ~0ull;
        const T* s = a + t * S;
        const uint8_t* w = where + t * S;
        for (int64_t base = blockIdx.x * span; any && base < S; base += (int64_t)gridDim.x * span) {
            T v[kMedianUnroll];
            bool ok[kMedianUnroll];
#pragma unroll
            for (int u = 0; u < kMedianUnroll; ++u) {
                const int64_t c = base + u * (int64_t)blockDim.x + threadIdx.x;
                ok[u] = c < S;
                if (ok[u]) {
                    v[u] = s[c];
                    ok[u] = !w[c];
                }
            }
#pragma unroll
            for (int u = 0; u < kMedianUnroll; ++u) {
                bool in = false;
                unsigned long long key = 0;
                if (ok[u] && !KT::is_nan(v[u])) {
                    key = KT::key(v[u]);
                    in = (key & mask) == prefix;
                    if (!in && key > prefix && key < my_above) my_above = key;
                }
                const unsigned m = __ballot_sync(0xffffffffu, in);
                if (m) {
                    const unsigned leader = __ffs(m) - 1;
                    unsigned long long slot = 0;
                    if (lane == leader) slot = atomicAdd(&cursor[t], (unsigned long long)__popc(m));
                    slot = __shfl_sync(0xffffffffu, slot, leader);
                    if (in) keys[out0 + slot + __popc(m & lt)] = key;
                }
            }
        }
        if (my_above != ~0ull) atomicMin(&above, my_above);
        __syncthreads();
        if (threadIdx.x == 0 && above != ~0ull) atomicMin(&st[t].min_above, above);
        __syncthreads();
    }
}

// candidates <= the lower median, and the smallest candidate above it
__global__ void median_upper_keys(const unsigned long long* __restrict__ keys, const int64_t* __restrict__ offsets,
                                  int64_t nt, MedianState* __restrict__ st) {
    __shared__ unsigned long long le, gt;
    for (int64_t t = blockIdx.y; t < nt; t += gridDim.y) {
        if (threadIdx.x == 0) {
            le = 0;
            gt = ~0ull;
        }
        __syncthreads();
        const unsigned long long lo = st[t].prefix;
        unsigned long long my_le = 0, my_gt = ~0ull;
        for (int64_t c = offsets[t] + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < offsets[t + 1];
             c += (int64_t)gridDim.x * blockDim.x) {
            const unsigned long long key = keys[c];
            if (key <= lo) ++my_le;
            else if (key < my_gt) my_gt = key;
        }
        if (my_le) atomicAdd(&le, my_le);
        if (my_gt != ~0ull) atomicMin(&gt, my_gt);
        __syncthreads();
        if (threadIdx.x == 0) {
            if (le) atomicAdd(&st[t].count_le, le);
            if (gt != ~0ull) atomicMin(&st[t].min_gt, gt);
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void median_write(const MedianState* __restrict__ st, int64_t nt, T* __restrict__ out) {
    using KT = Keys<T>;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const MedianState s = st[t];
    if (s.n == 0) {
        out[t] = T(0);
        return;
    }
    const T lo = KT::value((typename KT::K)s.prefix);
    if (s.n & 1) {
        out[t] = lo;
        return;
    }
    // the element after the lower median: itself when it repeats, else the
    // next candidate, else the first key above the candidate range
    const bool same = (unsigned long long)s.below + s.count_le >= (unsigned long long)(s.n / 2 + 1);
    const unsigned long long next = s.min_gt != ~0ull ? s.min_gt : s.min_above;
    out[t] = KT::mid(lo, same ? lo : KT::value((typename KT::K)next));
}

__global__ void median_init(MedianState* __restrict__ st, int64_t nt) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    st[t] = MedianState{0ull, 0ull, ~0ull, ~0ull, 0ull, 0, 0, 0, 0};
}

dim3 slice_grid(int64_t nt, int64_t S, int64_t per_block) {
    const int64_t ty = nt < 65535 ? nt : 65535;
    int64_t gx = (S + per_block - 1) / per_block;
    const int64_t cap = (6 * 152 + ty - 1) / ty;  // one wave of six 256-thread blocks per SM in all
    if (gx > cap) gx = cap;
    if (gx < 1) gx = 1;
    return dim3((unsigned)gx, (unsigned)(ty < 1 ? 1 : ty));
}

template <typename T>
int median_impl(const T* a, const uint8_t* where, int64_t nt, int64_t S, T* out, cudaStream_t s) {
    MedianState* st = nullptr;
    unsigned* hist = nullptr;
    int64_t* counts = nullptr;
    int64_t* offsets = nullptr;
    unsigned long long* cursor = nullptr;
    unsigned long long* keys = nullptr;
    int status = RG_OK;
    do {
        if ((status = dalloc(&st, nt, s))) break;
        if ((status = dalloc(&hist, nt * 256, s))) break;
        if ((status = dalloc(&counts, nt + 1, s))) break;
        if ((status = dalloc(&offsets, nt + 1, s))) break;
        if ((status = dalloc(&cursor, nt, s))) break;
        RG_CUDA(cudaMemsetAsync(hist, 0, nt * 256 * sizeof(unsigned), s));
        RG_CUDA(cudaMemsetAsync(cursor, 0, nt * sizeof(unsigned long long), s));
        const unsigned g1 = grid_for(nt, 256);
        const unsigned gw = grid_for(nt * 32, 256);  // a warp per slice
        median_init<<<g1, 256, 0, s>>>(st, nt);
        const dim3 grid = slice_grid(nt, S, 8192);
        constexpr int kPasses = Keys<T>::kBits / 8;
        for (int pass = 0; pass < kDataPasses; ++pass) {
            const int shift = Keys<T>::kBits - 8 * (pass + 1);
            median_hist<T><<<grid, 256, 0, s>>>(a, where, nt, S, shift, st, hist);
            median_pick<<<gw, 256, 0, s>>>(st, hist, nt, shift, pass);
        }
        // copy out the candidates (one host synchronisation for their count)
        median_cand_counts<<<grid_for(nt + 1, 256), 256, 0, s>>>(st, nt, counts);
        if ((status = exclusive_scan_i64(counts, offsets, nt + 1, nullptr, s))) break;
        int64_t total = 0;
        RG_CUDA(cudaMemcpyAsync(&total, offsets + nt, sizeof(total), cudaMemcpyDeviceToHost, s));
        RG_CUDA(cudaStreamSynchronize(s));
        if ((status = dalloc(&keys, total > 0 ? total : 1, s))) break;
        median_compact<T><<<grid, 256, 0, s>>>(a, where, nt, S, st, offsets, cursor, keys);
        const int64_t per_slice = (total + nt - 1) / (nt > 0 ? nt : 1);
        const dim3 kgrid = slice_grid(nt, per_slice, 4096);
        for (int pass = kDataPasses; pass < kPasses; ++pass) {
            const int shift = Keys<T>::kBits - 8 * (pass + 1);
            median_hist_keys<<<kgrid, 256, 0, s>>>(keys, offsets, nt, shift, st, hist);
            median_pick<<<gw, 256, 0, s>>>(st, hist, nt, shift, pass);
        }
        median_upper_keys<<<kgrid, 256, 0, s>>>(keys, offsets, nt, st);
        median_write<T><<<g1, 256, 0, s>>>(st, nt, out);
        RG_CUDA(cudaGetLastError());
    } while (0);
    dfree(keys, s);
    dfree(cursor, s);
    dfree(offsets, s);
    dfree(counts, s);
    dfree(hist, s);
    dfree(st, s);
    return status;
}

GsConst gs_constants(int64_t ny, int64_t nx) {
    // _iteration_gauss_seidel_2d (:121-129): the domain [-1, 1] on both axes
    GsConst k;
    const double dx = 2.0 / (double)(nx - 1);
    const double dy = 2.0 / (double)(ny - 1);
    k.dxxinv = 1.0 / (dx * dx);
    k.dyyinv = 1.0 / (dy * dy);
    k.dcent = 1.0 / (2.0 * (k.dxxinv + k.dyyinv));
    return k;
}

template <typename T>
int gauss_seidel_impl(T* a, const uint8_t* where, int64_t nt, int64_t ny, int64_t nx, const T* guess, int kind,
                      int64_t iterations, cudaStream_t s) {
    const int64_t S = ny * nx;
    T* med = nullptr;
    unsigned* counts = nullptr;
    int64_t* offsets = nullptr;
    int64_t* starts_dev = nullptr;
    uint64_t* list = nullptr;
    int status = RG_OK;
    do {
        // seed the missing cells
        if (kind == RG_FILL_GUESS_MEDIAN) {
            if ((status = dalloc(&med, nt, s))) break;
            if ((status = median_impl<T>(a, where, nt, S, med, s))) break;
            guess = med;
        }
        fill_seed<T><<<slice_grid(nt, S, 4096), 256, 0, s>>>(a, where, nt, S, guess, kind == RG_FILL_GUESS_FULL);
        RG_CUDA(cudaGetLastError());
        if (iterations == 0) break;

        // compact the missing cells of every (colour, phase) class
        const int64_t tiles = (S + kTile - 1) / kTile;
        const int64_t nblocks = nt * tiles;
        const int64_t ncounts = kClasses * nblocks + 1;
        if ((status = dalloc(&counts, ncounts, s))) break;
        if ((status = dalloc(&offsets, ncounts, s))) break;
        if ((status = dalloc(&starts_dev, kClasses + 1, s))) break;
        RG_CUDA(cudaMemsetAsync(counts, 0, ncounts * sizeof(unsigned), s));
        const dim3 cgrid((unsigned)tiles, (unsigned)(nt < 65535 ? nt : 65535));
        fill_count<<<cgrid, kClassifyThreads, 0, s>>>(where, nt, (uint32_t)ny, (uint32_t)nx, tiles, counts);
        if ((status = exclusive_scan_u32_to_i64(counts, offsets, ncounts, nullptr, s))) break;
        fill_class_starts<<<1, 32, 0, s>>>(offsets, nblocks, starts_dev);
        int64_t starts[kClasses + 1];
        RG_CUDA(cudaMemcpyAsync(starts, starts_dev, sizeof(starts), cudaMemcpyDeviceToHost, s));
        RG_CUDA(cudaStreamSynchronize(s));
        const int64_t total = starts[kClasses];
        if (total == 0) break;
        if ((status = dalloc(&list, total, s))) break;
        fill_lists<<<cgrid, kClassifyThreads, 0, s>>>(where, nt, (uint32_t)ny, (uint32_t)nx, tiles, offsets, list);
        RG_CUDA(cudaGetLastError());

        // relax: per iteration and colour, the phases in order (up to 16
        // blocks of 256 threads per SM: measured faster than one wave of
        // resident blocks, whose threads walk longer stretches of the list)
        const GsConst k = gs_constants(ny, nx);
        const FastDiv nx_div((uint32_t)nx);
        for (int64_t it = 0; it < iterations; ++it) {
            for (int cls = 0; cls < kClasses; ++cls) {
                const int64_t n = starts[cls + 1] - starts[cls];
                if (n == 0) continue;
                unsigned g = grid_for(n, 256);
                if (g > 152u * 16u) g = 152u * 16u;
                fill_update<T><<<g, 256, 0, s>>>(a, list + starts[cls], n, (uint32_t)ny, nx_div, k);
            }
        }
        RG_CUDA(cudaGetLastError());
    } while (0);
    dfree(list, s);
    dfree(starts_dev, s);
    dfree(offsets, s);
    dfree(counts, s);
    dfree(med, s);
    return status;
}

}  // namespace
}  // namespace rg

extern "C" int rg_fill_median(const void* d_a, int dtype, const uint8_t* d_where, int64_t nt, int64_t slice,
                              void* d_out, rg_stream_t stream) {
    rg::NvtxRange nvtx_range("rg_fill_median");
    using namespace rg;
    RG_CHECK(dtype == RG_F32 || dtype == RG_F64, RG_ERR_ARG, "rg_fill_median: dtype must be RG_F32 or RG_F64");
    RG_CHECK(nt >= 0 && slice >= 0, RG_ERR_ARG, "rg_fill_median: negative size");
    if (nt == 0) return RG_OK;
    RG_CHECK(d_out && (slice == 0 || (d_a && d_where)), RG_ERR_ARG, "rg_fill_median: NULL argument");
    cudaStream_t s = (cudaStream_t)stream;
    if (dtype == RG_F64) return median_impl<double>((const double*)d_a, d_where, nt, slice, (double*)d_out, s);
    return median_impl<float>((const float*)d_a, d_where, nt, slice, (float*)d_out, s);
}

extern "C" int rg_fill_gauss_seidel(void* d_a, int dtype, const uint8_t* d_where, int64_t nt, int64_t ny, int64_t nx,
                                    const void* d_guess, int guess_kind, int64_t iterations, rg_stream_t stream) {
    rg::NvtxRange nvtx_range("rg_fill_gauss_seidel");
    using namespace rg;
    RG_CHECK(dtype == RG_F32 || dtype == RG_F64, RG_ERR_ARG,
             "rg_fill_gauss_seidel: dtype must be RG_F32 or RG_F64");
    RG_CHECK(nt >= 0 && ny >= 0 && nx >= 0 && iterations >= 0, RG_ERR_ARG, "rg_fill_gauss_seidel: negative size");
    RG_CHECK(guess_kind == RG_FILL_GUESS_MEDIAN || guess_kind == RG_FILL_GUESS_SLICE ||
                 guess_kind == RG_FILL_GUESS_FULL,
             RG_ERR_ARG, "rg_fill_gauss_seidel: unknown guess kind %d", guess_kind);
    RG_CHECK(nt < (1ll << 31) && ny * nx < (1ll << 31), RG_ERR_ARG,
             "rg_fill_gauss_seidel: at most 2^31 slices of fewer than 2^31 cells");
    if (nt == 0 || ny * nx == 0) return RG_OK;
    RG_CHECK(iterations == 0 || (nx >= 2 && ny >= 2), RG_ERR_ARG,
             "rg_fill_gauss_seidel: division by zero (an axis of length 1)");
    RG_CHECK(d_a && d_where && (guess_kind == RG_FILL_GUESS_MEDIAN || d_guess), RG_ERR_ARG,
             "rg_fill_gauss_seidel: NULL argument");
    cudaStream_t s = (cudaStream_t)stream;
    if (dtype == RG_F64)
        return gauss_seidel_impl<double>((double*)d_a, d_where, nt, ny, nx, (const double*)d_guess, guess_kind,
                                         iterations, s);
    return gauss_seidel_impl<float>((float*)d_a, d_where, nt, ny, nx, (const float*)d_guess, guess_kind, iterations,
                                    s);
}
