// Warp-tiled apply: the float32 fast path of rg_apply.
//
// The plain kernel (apply.cu) gathers every input value straight from global
// memory; on a rotated grid the 32 gathers of a warp touch ~10 sectors spread
// over several input rows, so the L1 data pipe and instruction issue, not
// HBM, bound it.  Here every warp owns a compact 4 x 8 patch of output cells
// (a "warp tile", one cell per lane).  Once per weights matrix, each warp
// tile gets the sorted list of distinct 32-byte sectors (8 consecutive input
// cells) its rows read, and every stored entry gets the slot of its cell in
// that list.  The apply runs warp by warp with no block-wide
// synchronisation: for every group of 4 stack slices each lane loads one
// sector of the 4 slices with 128-bit loads (every fetched sector is one the
// tile needs), transposes it in registers and stores it to the warp's
// shared-memory stage interleaved by slice; each entry of a lane's row is
// then one 128-bit shared load that serves all 4 slices.  A second, scalar variant handles
// inputs whose slices are not 16-byte aligned.
#include "common.cuh"

namespace rg {
namespace {

constexpr int WARPS = 8;        // warp tiles per block
constexpr int TR = 4, TC = 8;   // warp tile: TR output rows x TC output columns
constexpr int PREP_MAX = 4096;  // entries of one warp tile sorted in shared memory
constexpr int CACHED_T = 8;     // row entries kept in registers across slices
constexpr int SLICES = 4;       // stack slices staged per step

struct TileShape {
    int64_t n0, n1;   // output shape (n0 = 1 when unknown)
    int64_t tr, tc;   // warp-tile extent (rows, columns)
    int64_t tiles1;   // warp tiles along axis 1
};

__device__ __forceinline__ int64_t row_of_lane(const TileShape& T, int64_t wt, int lane) {
    int64_t ti = wt / T.tiles1, tj = wt - ti * T.tiles1;
    int64_t i = ti * T.tr + lane / T.tc;
    int64_t j = tj * T.tc + lane % T.tc;
    if (i >= T.n0 || j >= T.n1) return -1;
    return i * T.n1 + j;
}

// Sort keys[0..n) ascending within one warp (bitonic over the next power of
// two, padded with INT32_MAX).
__device__ void warp_sort(int* keys, int n) {
    int lane = threadIdx.x & 31;
    int m = 1;
    while (m < n) m <<= 1;
    for (int q = n + lane; q < m; q += 32) keys[q] = INT32_MAX;
    __syncwarp();
    for (int k = 2; k <= m; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < m; i += 32) {
                int ixj = i ^ j;
                if (ixj > i) {
                    int a = keys[i], b = keys[ixj];
                    bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        keys[i] = b;
                        keys[ixj] = a;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// One warp per warp tile (blocks of 32 threads).  GRAIN 8 lists 32-byte
// sectors (key = column / 8, slot = the cell's float4 index in the vector
// kernel's stage); GRAIN 1 lists single cells (slot = position).  PASS 0 counts the list entries of the
// tile (0 when the tile has too many entries); PASS 1 writes the list from
// gptr[tile] and the slot of every entry.
template <int PASS, int GRAIN>
__global__ void __launch_bounds__(32)
    prepare_tiles(const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col, TileShape T,
                  int64_t* __restrict__ glen, const int64_t* __restrict__ gptr, int32_t* __restrict__ gidx,
                  uint16_t* __restrict__ slot) {
    __shared__ int keys[PREP_MAX];
    const int lane = threadIdx.x;
    const int64_t wt = blockIdx.x;
    const int64_t o = row_of_lane(T, wt, lane);
    int64_t s = 0, e = 0;
    if (o >= 0) {
        s = row_ptr[o];
        e = row_ptr[o + 1];
    }
    const int n = (int)(e - s);
    int incl = n;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += t;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    const int off = incl - n;
    if (total > PREP_MAX) {
        if (PASS == 0 && lane == 0) glen[wt] = 0;  // applied with direct gathers
        return;
    }
    for (int k = 0; k < n; k++) keys[off + k] = col[s + k] / GRAIN;
    __syncwarp();
    warp_sort(keys, total);
    // unique: every lane scans a contiguous slice of the sorted keys
    const int per = (total + 31) / 32;
    const int a0 = lane * per < total ? lane * per : total;
    const int a1 = a0 + per < total ? a0 + per : total;
    int cnt = 0;
    for (int i = a0; i < a1; i++) cnt += (i == 0) || (keys[i] != keys[i - 1]);
    int ci = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, ci, d);
        if (lane >= d) ci += t;
    }
    const int nu = __shfl_sync(0xffffffffu, ci, 31);
    if (PASS == 0) {
        if (lane == 0) glen[wt] = nu;
        return;
    }
    const int64_t g0 = gptr[wt];
    if (gptr[wt + 1] - g0 != nu) return;  // routed to the direct path
    int u = ci - cnt;
    for (int i = a0; i < a1; i++)
        if ((i == 0) || (keys[i] != keys[i - 1])) gidx[g0 + u++] = keys[i];
    __syncwarp();
    // slot of every entry of the lane's row (binary search in the sorted,
    // unique list just written)
    const int32_t* list = gidx + g0;
    for (int k = 0; k < n; k++) {
        const int c = col[s + k];
        const int key = c / GRAIN;
        int lo = 0, hi = nu - 1;
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (list[mid] < key) lo = mid + 1;
            else hi = mid;
        }
        if (GRAIN == 8) {
            // float4 index of the cell in the vector kernel's stage: half h
            // of the list, rotated by (h / 2) & 3
            const int h = 2 * lo + ((c & 7) >> 2);
            slot[s + k] = (uint16_t)(4 * h + (((c & 3) + (h >> 1)) & 3));
        } else {
            slot[s + k] = (uint16_t)lo;
        }
    }
}

__global__ void max_i64(const int64_t* a, int64_t n, unsigned long long* out) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        atomicMax(out, (unsigned long long)a[k]);
}

// Direct gathers for one lane's row (tiles whose list does not fit).
__device__ __forceinline__ void apply_direct(const int64_t s, const int64_t e, const int32_t* __restrict__ col,
                                             const float* __restrict__ val, const float* __restrict__ vin,
                                             int64_t n_in, float* out, int64_t n_out, int64_t d0, int64_t d1) {
    for (int64_t d = d0; d < d1; d++) {
        const float* a = vin + d * n_in;
        float acc = 0.f;
        for (int64_t k = s; k < e; k++) acc = fmaf(val[k], __ldg(a + col[k]), acc);
        out[d * n_out] = acc;
    }
}

// Vector variant: the list holds 32-byte sectors (8 cells, at most 32 per
// tile; longer lists take the scalar kernel).  A sector is fetched as two
// 16-byte halves, one per lane ("half h" = sector h / 2, half h % 2), so the
// 64 halves of a full list take two rounds of the warp.  Every lane loads its
// half for the 4 slices of the step (four 128-bit loads), transposes the
// 4 x 4 block in registers and stores cell i of the half as a float4 of the
// 4 slices at stage[4h + ((i + swz) & 3)], swz = (h / 2) & 3: the rotation
// spreads the 8 lanes of each store phase over distinct bank groups.  An
// entry's slot is that float4 index, so each entry of a lane's row costs one
// 128-bit shared load for all 4 slices.
__global__ void __launch_bounds__(32 * WARPS)
    apply_warp_vec(const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                   const uint16_t* __restrict__ slot, const float* __restrict__ val, TileShape T, int64_t n_wtiles,
                   const int64_t* __restrict__ gptr, const int32_t* __restrict__ gidx,
                   const float* __restrict__ vin, int64_t n_in, float* __restrict__ vout, int64_t n_out,
                   int64_t stack, int64_t chunk) {
    __shared__ float4 stage_all[WARPS][256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t wt = (int64_t)blockIdx.x * WARPS + warp;
    if (wt >= n_wtiles) return;
    float4* stage = stage_all[warp];
    const int64_t o = row_of_lane(T, wt, lane);
    const int64_t d0 = (int64_t)blockIdx.y * chunk;
    const int64_t d1 = d0 + chunk < stack ? d0 + chunk : stack;
    const int64_t g0 = gptr[wt];
    const int L = (int)(gptr[wt + 1] - g0);
    int64_t s = 0, e = 0;
    if (o >= 0) {
        s = row_ptr[o];
        e = row_ptr[o + 1];
    }
    const int nk = (int)(e - s);
    float* out = vout + (o >= 0 ? o : 0);
    if (L == 0 || L > 32) {
        if (o >= 0) apply_direct(s, e, col, val, vin, n_in, out, n_out, d0, d1);
        return;
    }
    // the two halves this lane fetches (rounds r = 0, 1), as float4 offsets
    // within a slice.  A lane without a half (past the list, or the second
    // half of a sector that starts past the end of the slice when n_in % 8
    // is 4) re-reads the first half of the list, which no slot refers to.
    bool has[2];
    int64_t src[2];
#pragma unroll
    for (int r = 0; r < 2; r++) {
        const int h = lane + 32 * r;
        const int64_t q = (h >> 1) < L ? (int64_t)gidx[g0 + (h >> 1)] * 2 + (h & 1) : -1;
        has[r] = q >= 0 && 4 * q < n_in;
        src[r] = has[r] ? q : (int64_t)gidx[g0] * 2;
    }
    const int swz = (lane >> 1) & 3;  // ((lane + 32 r) / 2) & 3 is the same for both rounds
    int li[CACHED_T];
    float w[CACHED_T];
#pragma unroll
    for (int k = 0; k < CACHED_T; k++) {
        li[k] = k < nk ? (int)slot[s + k] : 0;
        w[k] = k < nk ? val[s + k] : 0.f;
    }
    const float4* base = reinterpret_cast<const float4*>(vin);
    const int64_t row4 = n_in / 4;  // float4 per slice
    for (int64_t d = d0; d < d1; d += SLICES) {
        float4 v[2][SLICES];
#pragma unroll
        for (int r = 0; r < 2; r++) {
#pragma unroll
            for (int sl = 0; sl < SLICES; sl++) {
                const int64_t dd = d + sl < d1 ? d + sl : d;
                v[r][sl] = has[r] || r == 0 ? __ldg(base + dd * row4 + src[r]) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
        __syncwarp();  // the previous step's reads of the stage are done
#pragma unroll
        for (int r = 0; r < 2; r++) {
            if (r == 0 || has[r]) {
                float4* dst = stage + 4 * (lane + 32 * r);
                dst[(0 + swz) & 3] = make_float4(v[r][0].x, v[r][1].x, v[r][2].x, v[r][3].x);
                dst[(1 + swz) & 3] = make_float4(v[r][0].y, v[r][1].y, v[r][2].y, v[r][3].y);
                dst[(2 + swz) & 3] = make_float4(v[r][0].z, v[r][1].z, v[r][2].z, v[r][3].z);
                dst[(3 + swz) & 3] = make_float4(v[r][0].w, v[r][1].w, v[r][2].w, v[r][3].w);
            }
        }
        __syncwarp();
        if (o >= 0) {
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int k = 0; k < CACHED_T; k++) {
                if (k < nk) {
                    const float4 x = stage[li[k]];
                    acc.x = fmaf(w[k], x.x, acc.x);
                    acc.y = fmaf(w[k], x.y, acc.y);
                    acc.z = fmaf(w[k], x.z, acc.z);
                    acc.w = fmaf(w[k], x.w, acc.w);
                }
            }
            for (int64_t k = s + CACHED_T; k < e; k++) {
                const float wk = val[k];
                const float4 x = stage[slot[k]];
                acc.x = fmaf(wk, x.x, acc.x);
                acc.y = fmaf(wk, x.y, acc.y);
                acc.z = fmaf(wk, x.z, acc.z);
                acc.w = fmaf(wk, x.w, acc.w);
            }
            out[d * n_out] = acc.x;
            if (d + 1 < d1) out[(d + 1) * n_out] = acc.y;
            if (d + 2 < d1) out[(d + 2) * n_out] = acc.z;
            if (d + 3 < d1) out[(d + 3) * n_out] = acc.w;
        }
    }
}

// Scalar variant (slices not 16-byte aligned): single cells, PER per lane.
template <int PER>
__global__ void __launch_bounds__(32 * WARPS)
    apply_warp_scalar(const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                      const uint16_t* __restrict__ slot, const float* __restrict__ val, TileShape T,
                      int64_t n_wtiles, const int64_t* __restrict__ gptr, const int32_t* __restrict__ gidx,
                      const float* __restrict__ vin, int64_t n_in, float* __restrict__ vout, int64_t n_out,
                      int64_t stack, int64_t chunk) {
    constexpr int CELLS = 32 * PER;
    __shared__ float4 stage_all[WARPS][CELLS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t wt = (int64_t)blockIdx.x * WARPS + warp;
    if (wt >= n_wtiles) return;
    float* stage = reinterpret_cast<float*>(stage_all[warp]);
    const int64_t o = row_of_lane(T, wt, lane);
    const int64_t d0 = (int64_t)blockIdx.y * chunk;
    const int64_t d1 = d0 + chunk < stack ? d0 + chunk : stack;
    const int64_t g0 = gptr[wt];
    const int L = (int)(gptr[wt + 1] - g0);
    int64_t s = 0, e = 0;
    if (o >= 0) {
        s = row_ptr[o];
        e = row_ptr[o + 1];
    }
    const int nk = (int)(e - s);
    float* out = vout + (o >= 0 ? o : 0);
    if (L == 0 || L > CELLS) {
        if (o >= 0) apply_direct(s, e, col, val, vin, n_in, out, n_out, d0, d1);
        return;
    }
    int gl[PER];
#pragma unroll
    for (int p = 0; p < PER; p++) {
        const int q = lane + 32 * p;
        gl[p] = q < L ? gidx[g0 + q] : gidx[g0];
    }
    int li[CACHED_T];
    float w[CACHED_T];
#pragma unroll
    for (int k = 0; k < CACHED_T; k++) {
        li[k] = k < nk ? (int)slot[s + k] : 0;
        w[k] = k < nk ? val[s + k] : 0.f;
    }
    for (int64_t d = d0; d < d1; d += SLICES) {
        float r[SLICES][PER];
#pragma unroll
        for (int sl = 0; sl < SLICES; sl++) {
            const float* a = vin + (d + sl < d1 ? d + sl : d) * n_in;
#pragma unroll
            for (int p = 0; p < PER; p++) r[sl][p] = __ldg(a + gl[p]);
        }
        __syncwarp();
#pragma unroll
        for (int p = 0; p < PER; p++)
            reinterpret_cast<float4*>(stage)[lane + 32 * p] = make_float4(r[0][p], r[1][p], r[2][p], r[3][p]);
        __syncwarp();
        if (o >= 0) {
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int k = 0; k < CACHED_T; k++) {
                if (k < nk) {
                    const float4 v = reinterpret_cast<const float4*>(stage)[li[k]];
                    acc.x = fmaf(w[k], v.x, acc.x);
                    acc.y = fmaf(w[k], v.y, acc.y);
                    acc.z = fmaf(w[k], v.z, acc.z);
                    acc.w = fmaf(w[k], v.w, acc.w);
                }
            }
            for (int64_t k = s + CACHED_T; k < e; k++) {
                const float wk = val[k];
                const float4 v = reinterpret_cast<const float4*>(stage)[slot[k]];
                acc.x = fmaf(wk, v.x, acc.x);
                acc.y = fmaf(wk, v.y, acc.y);
                acc.z = fmaf(wk, v.z, acc.z);
                acc.w = fmaf(wk, v.w, acc.w);
            }
            out[d * n_out] = acc.x;
            if (d + 1 < d1) out[(d + 1) * n_out] = acc.y;
            if (d + 2 < d1) out[(d + 2) * n_out] = acc.z;
            if (d + 3 < d1) out[(d + 3) * n_out] = acc.w;
        }
    }
}

TileShape tile_shape(const rg_weights_s* W) {
    TileShape T;
    if (W->out_shape0 > 0 && W->out_shape1 > 0 && W->out_shape0 * W->out_shape1 == W->n_out) {
        T.n0 = W->out_shape0;
        T.n1 = W->out_shape1;
        T.tr = TR;
        T.tc = TC;
    } else {
        T.n0 = 1;
        T.n1 = W->n_out;
        T.tr = 1;
        T.tc = 32;
    }
    T.tiles1 = (T.n1 + T.tc - 1) / T.tc;
    return T;
}

}  // namespace

// Build the warp-tile lists of W for the given grain (8: 32-byte sectors for
// aligned inputs, 1: single cells), stream ordered, synchronising once.
// Called lazily by the first fast float32 apply of each kind.
int prepare_tiled(rg_weights_s* W, int grain, cudaStream_t s) {
    const int g = grain == 8 ? 1 : 0;
    if (W->tiled_ready[g]) return RG_OK;
    const TileShape T = tile_shape(W);
    const int64_t tiles = ((T.n0 + T.tr - 1) / T.tr) * T.tiles1;
    RG_CHECK(tiles < 0x7fffffff, RG_ERR_UNSUPPORTED, "apply: too many output tiles");
    int64_t* glen = nullptr;
    int64_t* total_dev = nullptr;
    unsigned long long* maxlen = nullptr;
    int st = RG_OK;
    do {
        if ((st = dalloc(&glen, (size_t)tiles + 1, s))) break;
        if ((st = dalloc(&maxlen, 1, s))) break;
        if ((st = dalloc(&W->t_gptr[g], (size_t)tiles + 1, s))) break;
        if ((st = dalloc(&total_dev, 1, s))) break;
        if ((st = dalloc(&W->t_slot[g], (size_t)W->nnz, s))) break;
        cudaMemsetAsync(glen + tiles, 0, sizeof(int64_t), s);
        if (grain == 8)
            prepare_tiles<0, 8><<<(unsigned)tiles, 32, 0, s>>>(W->row_ptr, W->col, T, glen, nullptr, nullptr,
                                                               nullptr);
        else
            prepare_tiles<0, 1><<<(unsigned)tiles, 32, 0, s>>>(W->row_ptr, W->col, T, glen, nullptr, nullptr,
                                                               nullptr);
        cudaMemsetAsync(maxlen, 0, sizeof(unsigned long long), s);
        max_i64<<<grid_for(tiles, 256) > 1024 ? 1024 : grid_for(tiles, 256), 256, 0, s>>>(glen, tiles, maxlen);
        if ((st = exclusive_scan_i64(glen, W->t_gptr[g], tiles + 1, total_dev, s))) break;
        int64_t total = 0;
        unsigned long long hmax = 0;
        cudaMemcpyAsync(&hmax, maxlen, sizeof(hmax), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(&total, total_dev, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("prepare_tiled: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }
        if ((st = dalloc(&W->t_gidx[g], (size_t)total, s))) break;
        if (grain == 8)
            prepare_tiles<1, 8><<<(unsigned)tiles, 32, 0, s>>>(W->row_ptr, W->col, T, nullptr, W->t_gptr[g],
                                                               W->t_gidx[g], W->t_slot[g]);
        else
            prepare_tiles<1, 1><<<(unsigned)tiles, 32, 0, s>>>(W->row_ptr, W->col, T, nullptr, W->t_gptr[g],
                                                               W->t_gidx[g], W->t_slot[g]);
        e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error("prepare_tiled: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }
        W->t_gmax[g] = (int)hmax;
        W->t_tiles = tiles;
        W->tiled_ready[g] = true;
    } while (0);
    dfree(glen, s);
    dfree(total_dev, s);
    dfree(maxlen, s);
    if (st) {
        dfree(W->t_gptr[g], s);
        dfree(W->t_gidx[g], s);
        dfree(W->t_slot[g], s);
        W->t_gptr[g] = nullptr;
        W->t_gidx[g] = nullptr;
        W->t_slot[g] = nullptr;
    }
    return st;
}

// Which lists the fast apply of `vin` uses (*g = 1: sector lists and the
// vector kernel; 0: cell lists and the scalar kernel), building them if they
// do not exist yet (*made set).  Sector lists need 16-byte aligned slices;
// when some tile's sector list exceeds 32 the cell lists are used instead.
// The caller holds the handle's lock.
int tiled_lists_for(rg_weights_s* W, const float* vin, cudaStream_t s, int* g, bool* made) {
    bool vec = W->n_in % 4 == 0 && ((uintptr_t)vin & 15) == 0;
    if (vec) {
        if (!W->tiled_ready[1]) *made = true;
        RG_TRY(prepare_tiled(W, 8, s));
        vec = W->t_gmax[1] <= 32;
    }
    if (!vec) {
        if (!W->tiled_ready[0]) *made = true;
        RG_TRY(prepare_tiled(W, 1, s));
    }
    *g = vec ? 1 : 0;
    return RG_OK;
}

int apply_tiled(const rg_weights_s* W, int g, const float* vin, float* vout, int64_t stack, cudaStream_t s) {
    const bool vec = g == 1;
    const TileShape T = tile_shape(W);
    const int64_t wtiles = W->t_tiles;
    const int64_t blocks = (wtiles + WARPS - 1) / WARPS;
    // slices per block: enough blocks for ~4 waves at 4 blocks per SM on 152
    // SMs, as many slices per block as that allows (a multiple of SLICES)
    const int64_t target_blocks = 152 * 4 * 4;
    int64_t chunks = (target_blocks + blocks - 1) / blocks;
    if (chunks < 1) chunks = 1;
    int64_t chunk = (stack + chunks - 1) / chunks;
    chunk = (chunk + SLICES - 1) / SLICES * SLICES;
    if ((stack + chunk - 1) / chunk > 65535) chunk = ((stack + 65534) / 65535 + SLICES - 1) / SLICES * SLICES;
    const int64_t nchunks = (stack + chunk - 1) / chunk;
    RG_CHECK(blocks < 0x7fffffff, RG_ERR_UNSUPPORTED, "apply: too many output tiles");
    dim3 grid((unsigned)blocks, (unsigned)nchunks);
    const int lmax = W->t_gmax[g];
#define RG_ARGS                                                                                               \
    W->row_ptr, W->col, W->t_slot[g], W->val32, T, wtiles, W->t_gptr[g], W->t_gidx[g], vin, W->n_in, vout, \
        W->n_out, stack, chunk
    if (vec) apply_warp_vec<<<grid, 32 * WARPS, 0, s>>>(RG_ARGS);
    else if (lmax <= 64) apply_warp_scalar<2><<<grid, 32 * WARPS, 0, s>>>(RG_ARGS);
    else if (lmax <= 128) apply_warp_scalar<4><<<grid, 32 * WARPS, 0, s>>>(RG_ARGS);
    else apply_warp_scalar<8><<<grid, 32 * WARPS, 0, s>>>(RG_ARGS);
#undef RG_ARGS
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

}  // namespace rg
