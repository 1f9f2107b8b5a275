// Staged applies: the float32 fast path of rg_apply and the exact float64
// apply of float32 stacks.
//
// The plain kernel (apply.cu) gathers every input value straight from global
// memory; on a rotated grid the 32 gathers of a warp touch ~10 sectors spread
// over several input rows, so the L1 data pipe and instruction issue, not
// HBM, bound it.  The kernels here stage input in shared memory first:
//
// * apply_patch_tma (input grid shape known): a block of 8 warps owns a
//   16 x 16 patch of output cells; tensor-map copies (TMA) bring the patch's
//   input box for a few slices at a time into a ring of stages behind
//   full/empty mbarriers; lanes gather from shared memory in a bank-aware
//   order.  Its EXACT form reproduces the upstream float64 sums bit for bit.
// * apply_rows (short input axis, long stacks): whole slices by 1D bulk
//   copies, entries held in registers.
// * apply_warp_vec / apply_warp_scalar (no shapes): every warp owns a 4 x 8
//   patch, loads the sorted list of input sectors its rows read with 128-bit
//   loads and restages it interleaved by slice, so that each entry is one
//   128-bit shared load serving 4 slices (the scalar form for unaligned
//   slices).
#include <cuda.h>  // CUtensorMap and its enums; the encoder comes from the runtime's driver entry point

#include <algorithm>
#include <climits>
#include <map>
#include <tuple>
#include <cstdio>
#include <cstdlib>

#include "common.cuh"

namespace rg {
namespace {

constexpr int WARPS = 8;        // warp tiles per block
constexpr int TR = 4, TC = 8;   // warp tile: TR output rows x TC output columns
constexpr int PREP_MAX = 1024;  // entries of one warp tile sorted in shared memory (4 KB per warp)
constexpr int CACHED_T = 8;     // row entries kept in registers across slices
constexpr int FF_EXTRA = 3;     // compensated mode: further row entries kept in shared memory
constexpr int ROW_EXTRA = 2;    // fast and exact modes: further row entries kept in shared memory
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

// ---------------------------------------------------------------------------
// TMA variant.  A block of 8 warps owns a 16 x 16 patch of output cells
// (4 x 2 warp tiles of 4 x 8).  The input footprint of every patch lies in a
// box of box_rows x 32 input cells (the same box size for all patches, the
// origin per patch, its column a multiple of 4 so that a copy starts on a
// 16-byte boundary).  A ring of NST stages, each holding SPS slices of the
// patch's box, is filled by one 3D tensor copy per stage (columns x rows x
// slices) issued by thread 0 and completed by the stage's "full" mbarrier
// transaction count; every warp arrives on the stage's "empty" mbarrier when
// it has read the stage, and thread 0 waits for all 8 before refilling it.
// The copies run on the TMA unit, so the load/store pipe only carries the
// gathers of the reduction (one 32-bit shared load per entry and slice).
// Box rows are 128 bytes and written with the 128-byte swizzle (16-byte
// chunk c of row r lands at chunk c ^ (r & 7) of that row), which spreads
// the gathers of vertically neighbouring cells over different banks; the
// entries' slots carry the swizzle.  Waits are bounded: a copy that does not
// land sets FLAG_TIMEOUT and the block leaves after a bounded drain.
// ---------------------------------------------------------------------------

constexpr int PATCH = 16;      // output cells per patch side
constexpr int PATCH_WARPS = 8; // 4 x 2 warp tiles of 4 x 8
constexpr int PBOX_C = 32;     // box columns: one 128-byte swizzle span
constexpr int PBOX_MAX_R = 32; // box rows at most
constexpr int PLANE = PBOX_MAX_R * PBOX_C;  // floats of one slice's plane in a stage (4 KB)

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}
// try_wait with a suspend-time hint (ns): the thread sleeps instead of spinning
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(20000u)
        : "memory");
    return ok != 0;
}
// bounded wait: gives up after 2^16 polls (each suspends at most ~20 us)
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
    for (int it = 0; it < (1 << 16); it++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_load_3d(float* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

struct PatchGrid {
    int64_t n0, n1;     // output cells
    int64_t patches1;   // patches along axis 1
};

__device__ __forceinline__ int64_t patch_cell(const PatchGrid& P, int64_t p, int r, int c) {
    const int64_t pi = p / P.patches1, pj = p - pi * P.patches1;
    const int64_t i = pi * PATCH + r, j = pj * PATCH + c;
    return (i < P.n0 && j < P.n1) ? i * P.n1 + j : -1;
}

// One block of 256 threads per patch, a thread per output cell.  PASS 0:
// footprint (origin, extent) of every patch; PASS 1: patches that fit the
// box get their entries' swizzled slots, the others are marked for direct
// gathers (origin row -2).
template <int PASS>
__global__ void __launch_bounds__(256)
    prepare_patch(const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col, PatchGrid P, FastDiv nd,
                  int2* __restrict__ origin, int2* __restrict__ extent, unsigned* __restrict__ stats, int BR,
                  uint16_t* __restrict__ slot) {
    __shared__ int red[4][8];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int64_t p = blockIdx.x;
    const int64_t o = patch_cell(P, p, t / PATCH, t % PATCH);
    int64_t s = 0, e = 0;
    if (o >= 0) {
        s = row_ptr[o];
        e = row_ptr[o + 1];
    }
    if (PASS == 0) {
        int rmin = INT_MAX, rmax = -1, cmin = INT_MAX, cmax = -1;
        for (int64_t k = s; k < e; k++) {
            const int c = col[k];
            const int r = (int)nd.div((uint32_t)c), cc = c - r * (int)nd.d;
            rmin = min(rmin, r);
            rmax = max(rmax, r);
            cmin = min(cmin, cc);
            cmax = max(cmax, cc);
        }
        rmin = __reduce_min_sync(0xffffffffu, rmin);
        cmin = __reduce_min_sync(0xffffffffu, cmin);
        rmax = __reduce_max_sync(0xffffffffu, rmax);
        cmax = __reduce_max_sync(0xffffffffu, cmax);
        if (lane == 0) {
            red[0][warp] = rmin;
            red[1][warp] = cmin;
            red[2][warp] = rmax;
            red[3][warp] = cmax;
        }
        __syncthreads();
        if (t == 0) {
            for (int w = 1; w < 8; w++) {
                rmin = min(rmin, red[0][w]);
                cmin = min(cmin, red[1][w]);
                rmax = max(rmax, red[2][w]);
                cmax = max(cmax, red[3][w]);
            }
            if (rmax < 0) {
                origin[p] = make_int2(-1, -1);
                extent[p] = make_int2(0, 0);
            } else {
                const int c0 = cmin & ~3;
                origin[p] = make_int2(rmin, c0);
                extent[p] = make_int2(rmax - rmin + 1, cmax - c0 + 1);
                atomicMax(&stats[0], (unsigned)(rmax - rmin + 1));
                atomicMax(&stats[1], (unsigned)(cmax - c0 + 1));
            }
        }
        return;
    }
    const int2 org = origin[p];
    const int2 ext = extent[p];
    if (org.x < 0) return;
    if (ext.x > BR || ext.y > PBOX_C) {
        __syncthreads();  // every thread has read origin before it changes
        if (t == 0) {
            origin[p] = make_int2(-2, -2);
            atomicAdd(&stats[2], 1u);
        }
        return;
    }
    for (int64_t k = s; k < e; k++) {
        const int c = col[k];
        const int row = (int)nd.div((uint32_t)c);
        const int r = row - org.x, cc = c - row * (int)nd.d - org.y;
        slot[k] = (uint16_t)(r * PBOX_C + ((((cc >> 2) ^ (r & 7)) << 2) | (cc & 3)));
    }
}

// Box slot of input cell c (the slot prepare_patch gives it).
__device__ __forceinline__ int box_slot_of(int c, int2 org, FastDiv nd) {
    const int row = (int)nd.div((uint32_t)c);
    const int r = row - org.x, cc = c - row * (int)nd.d - org.y;
    return r * PBOX_C + ((((cc >> 2) ^ (r & 7)) << 2) | (cc & 3));
}

// The part of a float64 weight that its float32 rounding hi = (float)w
// misses, rounded to float32: w - hi is exact in double (hi is w rounded to
// 24 bits), and hi + lo carries 48 bits of w (|w - hi - lo| <= 2^-48 |w|).
__device__ __forceinline__ float weight_rest(double w, float hi) {
    return __double2float_rn(__dsub_rn(w, (double)hi));
}

// Order of every lane's entries in the TMA kernel.  At step k each lane of
// a warp gathers its k-th entry; two lanes whose cells are different words
// of the same shared-memory bank (slot mod 32; the per-slice swizzle phase
// flips every lane's bank alike) are served one after the other, while lanes
// reading the same word share one access.  One block per patch, its threads
// laid out as in the apply kernel that will read the order (perm null: the
// warp tiles of the fast kernel; else thread t takes patch cell perm[t], the
// row-length order of the compensated kernel).  Greedy, step by step and
// lane by lane in lane order, with one level of augmentation: each lane
// takes the first of its remaining entries whose word an earlier lane reads
// at this step, else the first whose bank no earlier lane uses; else, if one
// of its entries' banks is held by a single earlier lane that can move to
// another of its entries (a shared word or a free bank), that lane moves and
// this one takes the bank; else its first remaining entry.  (Neighbouring
// output cells share input cells, so shared words are common.  On the
// 1024^2 -> 768^2 weights, in a model of the gathers, accesses per step go
// 2.15 (stored order) -> 1.56 (greedy) -> 1.28 (with the augmentation) for
// the warp tiles and 2.68 -> 2.11 -> 1.65 for the row-length layout.)  A
// lane's turn is taken by the whole warp: lane c tests the lane's candidate
// c, ballots give the pick, and the step's picks are written at its end.  The entries' natural slots come from
// slot_in, or from their columns when it is null; writes the reordered
// slots, float32 weights and (lo_out non-null) the weights' float32 rests.
// The CSR itself, which fixes the exact paths' order, is unchanged.  Lanes
// with more than ORDER_MAX entries keep the stored order.
constexpr int ORDER_MAX = 16;

__global__ void __launch_bounds__(32 * PATCH_WARPS)
    order_patch(const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col, FastDiv nd,
                const float* __restrict__ val32, const double* __restrict__ val, PatchGrid P,
                const int2* __restrict__ origin, const uint8_t* __restrict__ perm, const uint16_t* slot_in,
                uint16_t* slot_out, float* __restrict__ hi_out, float* __restrict__ lo_out) {
    __shared__ uint16_t cand[PATCH_WARPS][32][ORDER_MAX];  // every lane's natural slots
    __shared__ uint16_t owner[PATCH_WARPS][32];            // the word each bank serves at this step
    __shared__ int8_t owner_lane[PATCH_WARPS][32];          // the lane that holds the bank (first to take it)
    __shared__ uint8_t owner_cnt[PATCH_WARPS][32];          // lanes reading the bank's word
    __shared__ int8_t pick_of[PATCH_WARPS][32];             // every lane's candidate at this step
    __shared__ unsigned left_of[PATCH_WARPS][32];           // every lane's entries not yet placed
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int64_t p = blockIdx.x;
    int pr = 4 * (warp >> 1) + (lane >> 3), pc = 8 * (warp & 1) + (lane & 7);
    if (perm) {
        const int raw = perm[p * (PATCH * PATCH) + t];
        pr = raw / PATCH;
        pc = raw % PATCH;
    }
    const int64_t o = patch_cell(P, p, pr, pc);
    int64_t s = 0, e = 0;
    if (o >= 0) {
        s = row_ptr[o];
        e = row_ptr[o + 1];
    }
    const int nk = (int)(e - s);
    const int2 org = origin[p];
    if (org.x < 0) return;  // block-uniform
    auto natural = [&](int64_t k) -> uint16_t {
        return slot_in ? slot_in[k] : (uint16_t)box_slot_of(col[k], org, nd);
    };
    if (nk > ORDER_MAX) {
        for (int64_t k = s; k < e; k++) {
            slot_out[k] = natural(k);
            hi_out[k] = val32[k];
            if (lo_out) lo_out[k] = weight_rest(val[k], val32[k]);
        }
        // keep the stored order, but the other lanes still take part below
    }
    const int mine = nk <= ORDER_MAX ? nk : 0;
    for (int c = 0; c < mine; c++) cand[warp][lane][c] = natural(s + c);
    unsigned left = mine ? ((1u << mine) - 1u) : 0u;  // entries not yet placed (mine <= 16)
    const int kmax = __reduce_max_sync(0xffffffffu, mine);
    __syncwarp();
    const int c = lane & (ORDER_MAX - 1);  // the candidate this lane tests at each turn
    for (int k = 0; k < kmax; k++) {
        owner[warp][lane] = 0xffffu;
        owner_lane[warp][lane] = -1;
        owner_cnt[warp][lane] = 0;
        pick_of[warp][lane] = -1;
        left_of[warp][lane] = left;
        __syncwarp();
        for (int l = 0; l < 32; l++) {
            const unsigned lleft = left_of[warp][l];
            if (lleft == 0u) continue;  // warp-uniform
            bool share = false, freeb = false;
            uint16_t w = 0xffffu;
            if (lane < ORDER_MAX && ((lleft >> c) & 1u)) {
                w = cand[warp][l][c];
                const uint16_t ow = owner[warp][w & 31];
                share = ow == w;
                freeb = ow == 0xffffu;
            }
            const unsigned ms = __ballot_sync(0xffffffffu, share), mf = __ballot_sync(0xffffffffu, freeb);
            int pick = ms ? __ffs(ms) - 1 : (mf ? __ffs(mf) - 1 : -1);
            if (pick < 0) {
                // one level of augmentation: candidate c's bank is held by a
                // single lane m that can move to another of its entries
                int alt = -1, m = -1;
                if (w != 0xffffu) {
                    const int b = w & 31;
                    if (owner_cnt[warp][b] == 1) {
                        m = owner_lane[warp][b];
                        const uint16_t cur = owner[warp][b];
                        const unsigned mleft = left_of[warp][m];
                        for (int x = 0; x < ORDER_MAX && alt < 0; x++) {
                            if (!((mleft >> x) & 1u)) continue;
                            const uint16_t xw = cand[warp][m][x];
                            if (xw == cur) continue;
                            const uint16_t ox = owner[warp][xw & 31];
                            if (ox == xw || ox == 0xffffu) alt = x;
                        }
                    }
                }
                const unsigned ma = __ballot_sync(0xffffffffu, alt >= 0);
                if (ma) {
                    const int cs = __ffs(ma) - 1;
                    const int ms2 = __shfl_sync(0xffffffffu, m, cs), alt2 = __shfl_sync(0xffffffffu, alt, cs);
                    if (lane == 0) {
                        // lane ms2 moves to its entry alt2; lane l takes the freed bank
                        const uint16_t xw = cand[warp][ms2][alt2];
                        const uint16_t lw = cand[warp][l][cs];
                        pick_of[warp][ms2] = (int8_t)alt2;
                        if (owner[warp][xw & 31] == 0xffffu) {
                            owner[warp][xw & 31] = xw;
                            owner_lane[warp][xw & 31] = (int8_t)ms2;
                            owner_cnt[warp][xw & 31] = 1;
                        } else {
                            owner_cnt[warp][xw & 31]++;
                        }
                        owner[warp][lw & 31] = lw;
                        owner_lane[warp][lw & 31] = (int8_t)l;
                        owner_cnt[warp][lw & 31] = 1;
                        pick_of[warp][l] = (int8_t)cs;
                    }
                    __syncwarp();
                    continue;
                }
                pick = __ffs(lleft) - 1;
            }
            if (lane == 0) {
                const uint16_t pw = cand[warp][l][pick];
                const int b = pw & 31;
                if (owner[warp][b] == 0xffffu) {
                    owner[warp][b] = pw;
                    owner_lane[warp][b] = (int8_t)l;
                    owner_cnt[warp][b] = 1;
                } else if (owner[warp][b] == pw) {
                    owner_cnt[warp][b]++;
                }
                pick_of[warp][l] = (int8_t)pick;
            }
            __syncwarp();
        }
        // the step's picks
        const int pick = pick_of[warp][lane];
        if (pick >= 0) {
            left &= ~(1u << pick);
            slot_out[s + k] = cand[warp][lane][pick];
            hi_out[s + k] = val32[s + pick];
            if (lo_out) lo_out[s + k] = weight_rest(val[s + pick], val32[s + pick]);
        }
        __syncwarp();
    }
}

// Per patch, the threads' outputs for the exact and compensated applies: the
// patch's cells sorted by row length, longest first, so the 32 lanes of a
// warp run chains of similar length.  Lengths are compared in classes of
// `group` (1: exact lengths; the compensated apply takes classes of 3, which
// keeps more of a warp's cells near each other, so that more lanes share
// input words, for a little more divergence); ties by cell.  A bitonic sort
// of 256 keys in shared memory; one block per patch.
__global__ void __launch_bounds__(PATCH * PATCH)
    perm_patch(const int64_t* __restrict__ row_ptr, PatchGrid P, int group, uint8_t* __restrict__ perm) {
    __shared__ unsigned key[PATCH * PATCH];
    const int t = threadIdx.x;
    const int64_t p = blockIdx.x;
    const int64_t o = patch_cell(P, p, t / PATCH, t % PATCH);
    int64_t nk = o >= 0 ? row_ptr[o + 1] - row_ptr[o] : 0;
    if (nk > 255) nk = 255;
    key[t] = ((unsigned)((255 - nk) / group) << 8) | (unsigned)t;
    __syncthreads();
    for (int k = 2; k <= PATCH * PATCH; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            const int ixj = t ^ j;
            if (ixj > t) {
                const bool up = (t & k) == 0;
                const unsigned a = key[t], b = key[ixj];
                if ((a > b) == up) {
                    key[t] = b;
                    key[ixj] = a;
                }
            }
            __syncthreads();
        }
    }
    perm[p * (PATCH * PATCH) + t] = (uint8_t)(key[t] & 255u);
}

// Whether a float32 is finite, from its exponent bits.
__device__ __forceinline__ bool finite_bits(float f) {
    return (__float_as_uint(f) & 0x7f800000u) != 0x7f800000u;
}

// Whether a float32 is normal (neither zero, subnormal, infinite nor NaN).
__device__ __forceinline__ bool normal_bits(unsigned u) {
    return (u & 0x7f800000u) - 0x00800000u < 0x7f000000u;
}

// widen() of a normal float32, from its bits: the double's high word is the
// sign, the exponent rebiased by 1023 - 127 and the top 20 fraction bits;
// the low word the last 3 fraction bits.
__device__ __forceinline__ double widen_normal(unsigned u) {
    const unsigned hi = (u & 0x80000000u) | (((u & 0x7fffffffu) >> 3) + ((1023u - 127u) << 20));
    return __hiloint2double((int)hi, (int)(u << 29));
}

// Accumulation modes of the TMA apply.
//  MODE_FAST:  float32 output, acc = fmaf(w, x, acc) with float32 weights in
//              the bank-aware gather order.
//  MODE_EXACT: the upstream float64 apply bit for bit (float32 input, float64
//              weights and output): every entry in stored (CSR) order as
//              acc = acc + w * (double)x with one rounding per operation, from 0.0.
//  MODE_FF:    float64 output from float-float arithmetic on the FP32 pipe
//              (the GB300 runs FP32 at 64x its FP64 rate): each weight as
//              hi + lo floats, each product x * hi split exactly into p + e
//              by an FMA (Dekker's product), the running sum kept as an
//              unevaluated pair (h, l) with Knuth's two-sum, and h + l added
//              in double once per output.  Entries in the gather order.
constexpr int MODE_FAST = 0, MODE_EXACT = 1, MODE_FF = 2;

// Packed pairs of float32 (two slices of one output): the sm_100-family
// f32x2 instructions apply one IEEE operation, rounded to nearest, to both
// halves, at the issue cost of one scalar instruction.
__device__ __forceinline__ uint64_t f2_pack(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float2 f2_unpack(uint64_t v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f2_sub(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f2_mul(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// One float-float step on a pair of slices: (h, l) += x * (wh + wl), with
// the weight given as the pairs wh, -wh and wl.  Per half the operations
// and their results are those of the scalar step
//     p = x wh;  e = fma(x, wh, -p);  r = fma(x, wl, e);
//     t = h + p;  bp = t - h;  err = (h - (t - bp)) + (p - bp);
//     h = t;  l = l + (err + r)
// (Dekker's product, Knuth's two-sum), written with pn = x (-wh) = -p so
// that no operand needs negating: fma(x, wh, pn) = x wh - p, h - pn = h + p,
// and p - bp = -(pn + bp), subtracted from h - (t - bp).  (The only
// difference is the sign of an exact zero p - bp, which cannot reach the
// sum: h - (t - bp) is never -0, as h starts at +0.)
__device__ __forceinline__ void ff_step2(uint64_t& h, uint64_t& l, uint64_t wh, uint64_t whn, uint64_t wl,
                                         uint64_t x) {
    const uint64_t pn = f2_mul(x, whn);
    const uint64_t e = f2_fma(x, wh, pn);
    const uint64_t r = f2_fma(x, wl, e);
    const uint64_t t = f2_sub(h, pn);
    const uint64_t bp = f2_sub(t, h);
    const uint64_t err = f2_sub(f2_sub(h, f2_sub(t, bp)), f2_add(pn, bp));
    h = t;
    l = f2_add(l, f2_add(err, r));
}

template <int SPS, int NST, int MINB, int MODE, int CT = CACHED_T>
__global__ void __launch_bounds__(32 * PATCH_WARPS, MINB)
    apply_patch_tma(const __grid_constant__ CUtensorMap tmap, const int64_t* __restrict__ row_ptr,
                    const int32_t* __restrict__ col, const uint16_t* __restrict__ slot,
                    const float* __restrict__ bval, const float* __restrict__ blo, const float* __restrict__ val,
                    const double* __restrict__ dval, double* __restrict__ vout64, FastDiv nd,
                    PatchGrid P, int64_t n_patches, const int2* __restrict__ origin, int BR, int stage_floats,
                    unsigned box_bytes, const float* __restrict__ vin, int64_t n_in, float* __restrict__ vout,
                    int64_t n_out, int64_t stack, int64_t chunk, unsigned* __restrict__ flags,
                    const uint8_t* __restrict__ perm) {
    constexpr bool EXACT = MODE == MODE_EXACT;
    constexpr bool OUT64 = MODE != MODE_FAST;
    // The float64-output modes give every slice of a stage its own 4 KB plane
    // (constant gather offsets; one box copy per slice) and let the last warp
    // done with a stage refill it.  The float32 mode, whose gathers are few
    // instructions, keeps one box copy per stage (slices packed BR rows
    // apart) and a producer thread that waits for the warps; measured faster
    // for it.
    constexpr bool PLANES = MODE != MODE_FAST;
    __shared__ __align__(8) uint64_t full[NST], empty[NST];
    __shared__ unsigned done[NST];  // warps done with each stage, counted over all its uses
    // entries CT .. CT + NX - 1 of every thread's row, read once per patch
    // (rows one or two entries longer than the registers hold are common;
    // reading those entries from global memory at every stage held back the
    // warp with the longest rows, and with it the stage's refill): their
    // slots, and their float32 weights (fast), float32 weight and rest
    // (compensated) or float64 weights (exact)
    constexpr int NX = CT > 0 ? (MODE == MODE_FF ? FF_EXTRA : ROW_EXTRA) : 1;
    constexpr int NXF = MODE != MODE_EXACT ? NX : 1, NXL = MODE == MODE_FF ? NX : 1;
    constexpr int NXD = MODE == MODE_EXACT ? NX : 1;
    __shared__ uint16_t ex_slot[NX][32 * PATCH_WARPS];
    __shared__ float ex_hi[NXF][32 * PATCH_WARPS], ex_lo[NXL][32 * PATCH_WARPS];
    __shared__ double ex_d[NXD][32 * PATCH_WARPS];
    extern __shared__ __align__(1024) float ring[];
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int64_t p = blockIdx.x;
    // the thread's output: the warp tile layout, or for the exact and
    // compensated applies the patch's outputs by row length (a warp's lanes
    // then run chains of similar length)
    const int64_t d0 = (int64_t)blockIdx.y * chunk;
    const int64_t d1 = d0 + chunk < stack ? d0 + chunk : stack;
    const int2 org = origin[p];
    const int64_t ngroups = (d1 - d0 + SPS - 1) / SPS;
    // PLANES: one box copy per slice of the group (slices past the chunk are
    // not loaded); else one copy of box_bytes for the whole stage
    auto issue = [&](int st, int64_t grp) {
        const int64_t z0 = d0 + grp * SPS;
        if constexpr (PLANES) {
            const int n = (int)(d1 - z0 < SPS ? d1 - z0 : SPS);
            mbar_expect_tx(&full[st], (unsigned)n * box_bytes);
            for (int q = 0; q < n; q++)
                tma_load_3d(ring + (int64_t)st * stage_floats + q * PLANE, &tmap, org.y, org.x, (int)(z0 + q),
                            &full[st]);
        } else {
            mbar_expect_tx(&full[st], box_bytes);
            tma_load_3d(ring + (int64_t)st * stage_floats, &tmap, org.y, org.x, (int)z0, &full[st]);
        }
    };
    // the first stages' copies start before the threads fetch their rows, so
    // that the copies and the row fetches overlap (the barriers are ready for
    // the other threads after the __syncthreads below)
    if (org.x >= 0 && t == 0) {
        for (int k = 0; k < NST; k++) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], PATCH_WARPS);
            done[k] = 0u;
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        for (int k = 0; k < NST && k < ngroups; k++) issue(k, k);
    }
    int pr = 4 * (warp >> 1) + (lane >> 3), pc = 8 * (warp & 1) + (lane & 7);
    if (OUT64 && perm) {
        const int raw = perm[p * (PATCH * PATCH) + t];
        pr = raw / PATCH;
        pc = raw % PATCH;
    }
    const int64_t o = patch_cell(P, p, pr, pc);
    int64_t s = 0, e = 0;
    if (o >= 0) {
        s = row_ptr[o];
        e = row_ptr[o + 1];
    }
    const int nk = (int)(e - s);
    float* out = vout + (o >= 0 ? o : 0);
    if (org.x < 0) {
        // no entries (all zeros) or a footprint larger than the box: the whole block
        if (o >= 0) {
            if constexpr (OUT64) {
                for (int64_t d = d0; d < d1; d++) {
                    const float* a = vin + d * n_in;
                    double acc = 0.0;
                    for (int64_t k = s; k < e; k++) acc = __dadd_rn(acc, __dmul_rn(dval[k], (double)__ldg(a + col[k])));
                    vout64[d * n_out + o] = acc;
                }
            } else {
                apply_direct(s, e, col, val, vin, n_in, out, n_out, d0, d1);
            }
        }
        return;
    }
    // The compensated apply runs every lane of a warp to the warp's longest
    // row (a uniform bound, no divergent branch per entry).  A lane's entries
    // past its own row have zero weights and slot 0: such a step leaves the
    // pair (h, l) unchanged for a finite input word; a non-finite one makes
    // the sum NaN, which sends that output and slice to the exact loop.
    const int kwarp = MODE == MODE_FF ? __reduce_max_sync(0xffffffffu, nk) : nk;
    // PLANES: every slice of a stage has its own 4 KB plane, 1024-byte
    // aligned, so all slices see the same swizzle phase and a gather's
    // slices differ by constant offsets.  Otherwise the rows of slice q start
    // at row q * BR of the swizzle pattern: with BR a multiple of 4, odd
    // slices see the pattern shifted by 4 rows, which is the chunk index
    // xor 4 (slot xor 16).
    const int plane = PLANES ? PLANE : BR * PBOX_C;
    const int flip = PLANES ? 0 : ((BR & 4) ? 16 : 0);
    // (CT = 0 keeps a single dummy slot: every entry is read from memory)
    int li[CT > 0 ? CT : 1];
    float w[CT > 0 ? CT : 1];
    double wd[CT > 0 ? CT : 1];
    // the compensated mode's weights as packed pairs (wh, wh), (-wh, -wh), (wl, wl)
    uint64_t fh[CT > 0 ? CT : 1], fhn[CT > 0 ? CT : 1], fl[CT > 0 ? CT : 1];
#pragma unroll
    for (int k = 0; k < CT; k++) {
        if constexpr (EXACT) {
            li[k] = k < nk ? box_slot_of(col[s + k], org, nd) : 0;
            wd[k] = k < nk ? dval[s + k] : 0.0;
            w[k] = 0.f;
        } else if constexpr (MODE == MODE_FF) {
            li[k] = k < nk ? (int)slot[s + k] : 0;
            const float a = k < nk ? bval[s + k] : 0.f, b = k < nk ? blo[s + k] : 0.f;
            fh[k] = f2_pack(a, a);
            fhn[k] = f2_pack(-a, -a);
            fl[k] = f2_pack(b, b);
        } else {
            li[k] = k < nk ? (int)slot[s + k] : 0;
            w[k] = k < nk ? bval[s + k] : 0.f;
            wd[k] = 0.0;
        }
    }
    if constexpr (CT > 0) {
#pragma unroll
        for (int j = 0; j < NX; j++) {
            const bool has = CT + j < nk;
            if constexpr (EXACT) {
                ex_slot[j][t] = has ? (uint16_t)box_slot_of(col[s + CT + j], org, nd) : (uint16_t)0;
                ex_d[j][t] = has ? dval[s + CT + j] : 0.0;
            } else {
                ex_slot[j][t] = has ? slot[s + CT + j] : (uint16_t)0;
                ex_hi[j][t] = has ? bval[s + CT + j] : 0.f;
                if constexpr (MODE == MODE_FF) ex_lo[j][t] = has ? blo[s + CT + j] : 0.f;
            }
        }
    }
    __syncthreads();
    for (int64_t grp = 0; grp < ngroups; grp++) {
        const int st = (int)(grp % NST);
        const unsigned ph = (unsigned)((grp / NST) & 1);
        const bool got = mbar_wait_bounded(&full[st], ph);
        if (!__all_sync(0xffffffffu, got)) {
            if (lane == 0) {
                atomicOr(flags, FLAG_TIMEOUT);
                // copies of this block that may still be in flight: bounded wait before leaving
                for (int64_t q = grp + 1; q < grp + NST && q < ngroups; q++)
                    (void)mbar_wait_bounded(&full[q % NST], (unsigned)((q / NST) & 1));
            }
            return;
        }
        const float* buf = ring + (int64_t)st * stage_floats;
        const int64_t ds = d0 + grp * SPS;
        if constexpr (EXACT) {
            if (o >= 0) {
                double acc[SPS];
#pragma unroll
                for (int q = 0; q < SPS; q++) acc[q] = 0.0;
#pragma unroll
                for (int k = 0; k < CT; k++) {
                    if (k < nk) {
#pragma unroll
                        for (int q = 0; q < SPS; q++)
                            acc[q] = __dadd_rn(
                                acc[q], __dmul_rn(wd[k], widen(buf[q * plane + (li[k] ^ ((q & 1) ? flip : 0))])));
                    }
                }
                if constexpr (CT > 0) {
#pragma unroll
                    for (int j = 0; j < NX; j++) {
                        if (CT + j < nk) {
                            const double wk = ex_d[j][t];
                            const int sk = ex_slot[j][t];
#pragma unroll
                            for (int q = 0; q < SPS; q++)
                                acc[q] = __dadd_rn(acc[q],
                                                   __dmul_rn(wk, widen(buf[q * plane + (sk ^ ((q & 1) ? flip : 0))])));
                        }
                    }
                }
                for (int64_t k = s + (CT > 0 ? CT + NX : 0); k < e; k++) {
                    const double wk = dval[k];
                    const int sk = box_slot_of(col[k], org, nd);
#pragma unroll
                    for (int q = 0; q < SPS; q++)
                        acc[q] = __dadd_rn(acc[q], __dmul_rn(wk, widen(buf[q * plane + (sk ^ ((q & 1) ? flip : 0))])));
                }
#pragma unroll
                for (int q = 0; q < SPS; q++)
                    if (ds + q < d1) vout64[(ds + q) * n_out + o] = acc[q];
            }
        } else if constexpr (MODE == MODE_FF) {
            if (o >= 0) {
                // slices 2j and 2j + 1 of the stage as one packed pair
                static_assert(SPS % 2 == 0, "the compensated apply stages slices in pairs");
                uint64_t h2[SPS / 2], l2[SPS / 2];
#pragma unroll
                for (int j = 0; j < SPS / 2; j++) h2[j] = l2[j] = 0ull;
#pragma unroll
                for (int k = 0; k < CT; k++) {
                    if (k < kwarp) {
                        const int a = li[k], b = li[k] ^ flip;
#pragma unroll
                        for (int j = 0; j < SPS / 2; j++)
                            ff_step2(h2[j], l2[j], fh[k], fhn[k], fl[k],
                                     f2_pack(buf[2 * j * plane + a], buf[(2 * j + 1) * plane + b]));
                    }
                }
                if constexpr (CT > 0) {
#pragma unroll
                    for (int j = 0; j < NX; j++) {
                        if (CT + j < kwarp) {
                            const float wk = ex_hi[j][t], wlk = ex_lo[j][t];
                            const uint64_t kh = f2_pack(wk, wk), khn = f2_pack(-wk, -wk), kl = f2_pack(wlk, wlk);
                            const int a = ex_slot[j][t], b = a ^ flip;
#pragma unroll
                            for (int q = 0; q < SPS / 2; q++)
                                ff_step2(h2[q], l2[q], kh, khn, kl,
                                         f2_pack(buf[2 * q * plane + a], buf[(2 * q + 1) * plane + b]));
                        }
                    }
                }
                for (int64_t k = s + (CT > 0 ? CT + NX : 0); k < e; k++) {
                    const float wk = bval[k], wlk = blo[k];
                    const uint64_t kh = f2_pack(wk, wk), khn = f2_pack(-wk, -wk), kl = f2_pack(wlk, wlk);
                    const int a = slot[k], b = a ^ flip;
#pragma unroll
                    for (int j = 0; j < SPS / 2; j++)
                        ff_step2(h2[j], l2[j], kh, khn, kl,
                                 f2_pack(buf[2 * j * plane + a], buf[(2 * j + 1) * plane + b]));
                }
                float h[SPS], l[SPS];
#pragma unroll
                for (int j = 0; j < SPS / 2; j++) {
                    const float2 hv = f2_unpack(h2[j]), lv = f2_unpack(l2[j]);
                    h[2 * j] = hv.x;
                    h[2 * j + 1] = hv.y;
                    l[2 * j] = lv.x;
                    l[2 * j + 1] = lv.y;
                }
                // The usual stage (every slice in range, every h and l a
                // normal float) is tested once, with bitwise ands and a single
                // branch, and stored without further tests (per-slice tests
                // and branches were a measured share of the instruction
                // stream).  Anything else takes the per-slice path.
                bool usual = ds + SPS <= d1;
#pragma unroll
                for (int q = 0; q < SPS; q++)
                    usual = usual & normal_bits(__float_as_uint(h[q])) & normal_bits(__float_as_uint(l[q]));
                if (usual) {
                    double* dst = vout64 + ds * n_out + o;
#pragma unroll
                    for (int q = 0; q < SPS; q++)
                        dst[q * n_out] =
                            __dadd_rn(widen_normal(__float_as_uint(h[q])), widen_normal(__float_as_uint(l[q])));
                } else {
#pragma unroll
                    for (int q = 0; q < SPS; q++) {
                        if (ds + q >= d1) continue;
                        double r;
                        const unsigned uh = __float_as_uint(h[q]), ul = __float_as_uint(l[q]);
                        if (normal_bits(uh) && normal_bits(ul)) {
                            r = __dadd_rn(widen_normal(uh), widen_normal(ul));
                        } else if (nk == 0) {
                            r = 0.0;
                        } else if (finite_bits(h[q]) && finite_bits(l[q])) {
                            r = __dadd_rn(widen(h[q]), widen(l[q]));
                        } else {
                            // a float32 partial sum overflowed, or an input or
                            // a weight is not finite (or a padded step read a
                            // non-finite word): this output and slice in
                            // float64, stored order (the exact apply's sum)
                            r = 0.0;
                            for (int64_t k = s; k < e; k++)
                                r = __dadd_rn(r, __dmul_rn(dval[k], widen(buf[q * plane + (box_slot_of(col[k], org, nd) ^
                                                                                         ((q & 1) ? flip : 0))])));
                        }
                        vout64[(ds + q) * n_out + o] = r;
                    }
                }
            }
        } else if (o >= 0) {
            float acc[SPS];
#pragma unroll
            for (int q = 0; q < SPS; q++) acc[q] = 0.f;
#pragma unroll
            for (int k = 0; k < CT; k++) {
                if (k < nk) {
#pragma unroll
                    for (int q = 0; q < SPS; q++)
                        acc[q] = fmaf(w[k], buf[q * plane + (li[k] ^ ((q & 1) ? flip : 0))], acc[q]);
                }
            }
            if constexpr (CT > 0) {
#pragma unroll
                for (int j = 0; j < NX; j++) {
                    if (CT + j < nk) {
                        const float wk = ex_hi[j][t];
                        const int sk = ex_slot[j][t];
#pragma unroll
                        for (int q = 0; q < SPS; q++)
                            acc[q] = fmaf(wk, buf[q * plane + (sk ^ ((q & 1) ? flip : 0))], acc[q]);
                    }
                }
            }
            for (int64_t k = s + (CT > 0 ? CT + NX : 0); k < e; k++) {
                const float wk = bval[k];
                const int sk = slot[k];
#pragma unroll
                for (int q = 0; q < SPS; q++) acc[q] = fmaf(wk, buf[q * plane + (sk ^ ((q & 1) ? flip : 0))], acc[q]);
            }
#pragma unroll
            for (int q = 0; q < SPS; q++)
                if (ds + q < d1) out[(ds + q) * n_out] = acc[q];
        }
        // The last warp done with the stage refills it, so no warp waits for
        // the others (the slowest warp, with the longest rows, no longer
        // holds a producer thread back).  Its lanes' reads of the stage are
        // ordered before the count (syncwarp, then a release fence); the last
        // one acquires them all before the async-proxy copy overwrites it.
        __syncwarp();
        if constexpr (PLANES) {
            if (lane == 0) {
                __threadfence_block();
                const unsigned n = atomicAdd(&done[st], 1u) + 1u;
                if (n == (unsigned)(grp / NST + 1) * PATCH_WARPS && grp + NST < ngroups) {
                    __threadfence_block();
                    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                    issue(st, grp + NST);
                }
            }
        } else {
            if (lane == 0) mbar_arrive(&empty[st]);  // this warp is done with the stage
            if (t == 0 && grp + NST < ngroups) {
                if (!mbar_wait_bounded(&empty[st], ph)) {
                    atomicOr(flags, FLAG_TIMEOUT);
                    for (int64_t q = grp + 1; q < grp + NST && q < ngroups; q++)
                        (void)mbar_wait_bounded(&full[q % NST], (unsigned)((q / NST) & 1));
                    return;
                }
                // the warps' generic-proxy reads of the stage before the async-proxy writes
                asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                issue(st, grp + NST);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Row variant, for weights with a short input axis (a whole slice fits in
// shared memory: 1D multilinear or conservative weights over many spectra).
// A persistent block of ROWS_THREADS threads walks slices d = blockIdx.x,
// blockIdx.x + gridDim.x, ...; thread 0 fills a ring of ROWS_NST stages with
// one 1D bulk copy per slice (cp.async.bulk, completed by the stage's full
// mbarrier); every thread keeps the entries of its outputs (o = t, t + T,
// ...; at most ROWS_E entries each) in registers, reduces them from shared
// memory and stores coalesced; warps release a stage on its empty mbarrier.
// ---------------------------------------------------------------------------

constexpr int ROWS_THREADS = 1024;
constexpr int ROWS_J = 4;   // outputs per thread (n_out <= ROWS_THREADS * ROWS_J)
constexpr int ROWS_E = 4;   // entries per output at most
constexpr int ROWS_NST = 3;

__device__ __forceinline__ void bulk_load(float* dst, const float* src, unsigned bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__global__ void __launch_bounds__(ROWS_THREADS, 1)
    apply_rows(const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col, const float* __restrict__ val,
               const float* __restrict__ vin, int64_t n_in, float* __restrict__ vout, int64_t n_out, int64_t stack,
               int stage_floats, unsigned* __restrict__ flags) {
    __shared__ __align__(8) uint64_t full[ROWS_NST], empty[ROWS_NST];
    extern __shared__ __align__(128) float rbuf[];
    const int t = threadIdx.x, lane = t & 31;
    constexpr int NWARPS = ROWS_THREADS / 32;
    int c[ROWS_J][ROWS_E];
    float w[ROWS_J][ROWS_E];
#pragma unroll
    for (int j = 0; j < ROWS_J; j++) {
        const int64_t o = t + (int64_t)j * ROWS_THREADS;
        int64_t s = 0, e = 0;
        if (o < n_out) {
            s = row_ptr[o];
            e = row_ptr[o + 1];
        }
#pragma unroll
        for (int k = 0; k < ROWS_E; k++) {
            c[j][k] = s + k < e ? col[s + k] : 0;
            w[j][k] = s + k < e ? val[s + k] : 0.f;
        }
    }
    if (t == 0) {
        for (int k = 0; k < ROWS_NST; k++) {
            mbar_init(&full[k], 1);
            mbar_init(&empty[k], NWARPS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    const unsigned bytes = (unsigned)(n_in * 4);
    // slices of this block: d = blockIdx.x + i * gridDim.x
    const int64_t nmine = blockIdx.x < stack ? (stack - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    auto issue = [&](int st, int64_t i) {
        mbar_expect_tx(&full[st], bytes);
        bulk_load(rbuf + (int64_t)st * stage_floats, vin + (blockIdx.x + i * gridDim.x) * n_in, bytes, &full[st]);
    };
    if (t == 0)
        for (int k = 0; k < ROWS_NST && k < nmine; k++) issue(k, k);
    for (int64_t i = 0; i < nmine; i++) {
        const int st = (int)(i % ROWS_NST);
        const unsigned ph = (unsigned)((i / ROWS_NST) & 1);
        const bool got = mbar_wait_bounded(&full[st], ph);
        if (!__all_sync(0xffffffffu, got)) {
            if (lane == 0) atomicOr(flags, FLAG_TIMEOUT);
            if (t == 0)
                for (int64_t q = i + 1; q < i + ROWS_NST && q < nmine; q++)
                    (void)mbar_wait_bounded(&full[q % ROWS_NST], (unsigned)((q / ROWS_NST) & 1));
            return;
        }
        const float* buf = rbuf + (int64_t)st * stage_floats;
        float* out = vout + (blockIdx.x + i * gridDim.x) * n_out;
#pragma unroll
        for (int j = 0; j < ROWS_J; j++) {
            const int64_t o = t + (int64_t)j * ROWS_THREADS;
            if (o < n_out) {
                float acc = 0.f;
#pragma unroll
                for (int k = 0; k < ROWS_E; k++) acc = fmaf(w[j][k], buf[c[j][k]], acc);
                out[o] = acc;
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[st]);
        if (t == 0 && i + ROWS_NST < nmine) {
            if (!mbar_wait_bounded(&empty[st], ph)) {
                atomicOr(flags, FLAG_TIMEOUT);
                for (int64_t q = i + 1; q < i + ROWS_NST && q < nmine; q++)
                    (void)mbar_wait_bounded(&full[q % ROWS_NST], (unsigned)((q / ROWS_NST) & 1));
                return;
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            issue(st, i + ROWS_NST);
        }
    }
}

// longest row of a CSR (atomicMax over rows)
__global__ void max_row_len(const int64_t* __restrict__ row_ptr, int64_t n, unsigned* __restrict__ out) {
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < n; o += (int64_t)gridDim.x * blockDim.x) {
        const int64_t len = row_ptr[o + 1] - row_ptr[o];
        atomicMax(out, (unsigned)(len > 0xffffffffll ? 0xffffffffll : len));
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, []() {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        cudaGetLastError();
    });
    return fn;
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
        small_to_host(&hmax, maxlen, sizeof(hmax), s);
        small_to_host(&total, total_dev, sizeof(int64_t), s);
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

// Whether the TMA apply can take this call: output and input grid shapes
// known, input rows of whole 16-byte chunks, 16-byte aligned slices.
bool box_usable(const rg_weights_s* W, const float* vin, int64_t stack) {
    return W->box_state >= 0 && W->out_shape0 > 0 && W->out_shape1 > 0 &&
           W->out_shape0 * W->out_shape1 == W->n_out && W->in_shape0 > 0 && W->in_shape1 > 0 &&
           W->in_shape1 % 4 == 0 && W->in_shape0 * W->in_shape1 == W->n_in && ((uintptr_t)vin & 15) == 0 &&
           stack >= 1 && W->n_in < INT32_MAX && stack < INT32_MAX && encode_tiled() != nullptr;
}

PatchGrid patch_grid(const rg_weights_s* W) {
    PatchGrid P;
    P.n0 = W->out_shape0;
    P.n1 = W->out_shape1;
    P.patches1 = (P.n1 + PATCH - 1) / PATCH;
    return P;
}

// Build the patch lists of W (the caller holds the handle's lock; *made set
// when anything was launched).  Leaves box_state -1 when the footprints do
// not fit a box (more than 1 % of the patches, and more than 4, would need
// direct gathers).
// The exact apply's per-patch thread order (made once, with the box lists).
int box_perm_for(rg_weights_s* W, cudaStream_t s, bool* made) {
    if (W->box_perm || W->box_state != 1) return RG_OK;
    *made = true;
    RG_TRY(dalloc(&W->box_perm, (size_t)W->box_patches * PATCH * PATCH, s));
    perm_patch<<<(unsigned)W->box_patches, PATCH * PATCH, 0, s>>>(W->row_ptr, patch_grid(W), 1, W->box_perm);
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

// The compensated apply's per-patch thread order (row lengths in classes of 3).
constexpr int FF_LENGTH_CLASS = 3;
int ff_perm_for(rg_weights_s* W, cudaStream_t s, bool* made) {
    if (W->ff_perm || W->box_state != 1) return RG_OK;
    *made = true;
    RG_TRY(dalloc(&W->ff_perm, (size_t)W->box_patches * PATCH * PATCH, s));
    perm_patch<<<(unsigned)W->box_patches, PATCH * PATCH, 0, s>>>(W->row_ptr, patch_grid(W), FF_LENGTH_CLASS,
                                                                  W->ff_perm);
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

// The compensated apply's entry order (made once, after the box lists):
// threads take the patch's outputs by row length (ff_perm), and every
// lane's entries are ordered for that layout with their float32 weights and
// the weights' float32 rests.
int ff_lists_for(rg_weights_s* W, cudaStream_t s, bool* made) {
    if (W->ff_slot || W->box_state != 1) return RG_OK;
    RG_TRY(ff_perm_for(W, s, made));
    *made = true;
    int st = RG_OK;
    do {
        if ((st = dalloc(&W->ff_slot, (size_t)W->nnz, s))) break;
        if ((st = dalloc(&W->ff_hi, (size_t)W->nnz, s))) break;
        if ((st = dalloc(&W->ff_lo, (size_t)W->nnz, s))) break;
        order_patch<<<(unsigned)W->box_patches, 32 * PATCH_WARPS, 0, s>>>(
            W->row_ptr, W->col, FastDiv((uint32_t)W->in_shape1), W->val32, W->val, patch_grid(W), W->box_origin, W->ff_perm, nullptr,
            W->ff_slot, W->ff_hi, W->ff_lo);
        if (cudaGetLastError() != cudaSuccess) {
            set_error("apply (compensated lists): launch failed");
            st = RG_ERR_CUDA;
        }
    } while (0);
    if (st != RG_OK) {
        dfree(W->ff_slot, s);
        dfree(W->ff_hi, s);
        dfree(W->ff_lo, s);
        W->ff_slot = nullptr;
        W->ff_hi = nullptr;
        W->ff_lo = nullptr;
    }
    return st;
}

int box_lists_for(rg_weights_s* W, cudaStream_t s, bool* made) {
    if (W->box_state != 0) return RG_OK;
    *made = true;
    const PatchGrid P = patch_grid(W);
    const int64_t patches = ((P.n0 + PATCH - 1) / PATCH) * P.patches1;
    RG_CHECK(patches < 0x7fffffff, RG_ERR_UNSUPPORTED, "apply: too many output patches");
    int2* extent = nullptr;
    unsigned* stats = nullptr;
    int st = RG_OK;
    do {
        if ((st = dalloc(&W->box_origin, (size_t)patches, s))) break;
        if ((st = dalloc(&extent, (size_t)patches, s))) break;
        if ((st = dalloc(&stats, 4, s))) break;
        if ((st = dalloc(&W->box_slot, (size_t)W->nnz, s))) break;
        if (W->dflags == nullptr) {
            if ((st = dalloc(&W->dflags, 1, s))) break;
            cudaMemsetAsync(W->dflags, 0, sizeof(unsigned), s);
        }
        cudaMemsetAsync(stats, 0, 4 * sizeof(unsigned), s);
        prepare_patch<0><<<(unsigned)patches, 256, 0, s>>>(W->row_ptr, W->col, P, FastDiv((uint32_t)W->in_shape1), W->box_origin,
                                                           extent, stats, 0, nullptr);
        unsigned h[4] = {0, 0, 0, 0};
        small_to_host(h, stats, sizeof(h), s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("apply (patch lists): %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }
        // box rows: a multiple of 4 (keeps the swizzle phase of every slice at 0 or 4)
        const int BR = (int)((std::min<unsigned>(std::max<unsigned>(h[0], 1u), PBOX_MAX_R) + 3) & ~3u);
        prepare_patch<1><<<(unsigned)patches, 256, 0, s>>>(W->row_ptr, W->col, P, FastDiv((uint32_t)W->in_shape1), W->box_origin,
                                                           extent, stats, BR, W->box_slot);
        small_to_host(h, stats, sizeof(h), s);
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("apply (patch lists): %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }
        W->box_rows = BR;
        W->box_cols = PBOX_C;
        W->box_patches = patches;
        const bool few = (int64_t)h[2] * 100 <= patches || h[2] <= 4;  // patches left to direct gathers
        W->box_state = few && BR <= W->in_shape0 && PBOX_C <= W->in_shape1 ? 1 : -1;
        if (W->box_state != 1) break;  // footprints too large for a box: no entry order needed
        if ((st = dalloc(&W->box_val, (size_t)W->nnz, s))) break;
        order_patch<<<(unsigned)patches, 32 * PATCH_WARPS, 0, s>>>(W->row_ptr, W->col, FastDiv((uint32_t)W->in_shape1),
                                                                   W->val32, W->val, P, W->box_origin, nullptr,
                                                                   W->box_slot, W->box_slot, W->box_val, nullptr);
    } while (0);
    dfree(extent, s);
    dfree(stats, s);
    if (st != RG_OK || W->box_state != 1) {
        dfree(W->box_origin, s);
        dfree(W->box_slot, s);
        dfree(W->box_val, s);
        W->box_origin = nullptr;
        W->box_slot = nullptr;
        W->box_val = nullptr;
        if (st == RG_OK) W->box_state = -1;
    }
    return st;
}

// Configurations of the TMA apply: slices per stage, stages, and the blocks
// per SM its registers are capped for (0: no cap).  The autotuner below
// times each on the first apply of a handle; RG_APPLY_BOX_CONFIG="sps,nst,minb"
// forces one.
struct BoxConfig {
    int sps, nst, minb;
};
constexpr BoxConfig kBoxConfigs[] = {{4, 2, 0}, {4, 2, 4}, {4, 3, 4}, {2, 3, 4}, {2, 4, 4}, {8, 2, 0}, {4, 3, 0}};
constexpr int kNumBoxConfigs = (int)(sizeof(kBoxConfigs) / sizeof(kBoxConfigs[0]));
// The compensated kernel's configurations add the number of entries a
// thread keeps in registers (fewer registers, more resident blocks); forced
// by RG_APPLY_FF_CONFIG="sps,nst,minb,cached".
struct FFConfig {
    int sps, nst, minb, cached;
};
constexpr FFConfig kFFConfigs[] = {{6, 2, 0, 6}, {8, 2, 0, 6}, {4, 2, 0, 6}, {4, 3, 0, 6},
                                   {2, 4, 0, 6}, {4, 3, 3, 4}, {4, 2, 4, 0}};
constexpr int kNumFFConfigs = (int)(sizeof(kFFConfigs) / sizeof(kFFConfigs[0]));

template <int SPS, int NST, int MINB, int MODE = MODE_FAST, int CT = CACHED_T>
int launch_patch(const rg_weights_s* W, const CUtensorMap& map, int box_slices, const float* vin, void* vout,
                 int64_t stack, cudaStream_t s) {
    const int BR = W->box_rows;
    // stages (and with planes, every slice) start on 1024-byte boundaries
    constexpr bool PLANES = MODE != MODE_FAST;
    const int stage_floats = PLANES ? SPS * PLANE : (SPS * BR * PBOX_C + 255) & ~255;
    const unsigned box_bytes = (unsigned)((PLANES ? 1 : box_slices) * BR * PBOX_C * 4);
    const size_t smem = (size_t)NST * stage_floats * sizeof(float);
    if (smem > 200 * 1024) return RG_ERR_UNSUPPORTED;
    static std::once_flag attr;
    std::call_once(attr, []() {
        cudaFuncSetAttribute(apply_patch_tma<SPS, NST, MINB, MODE, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             200 * 1024);
        cudaGetLastError();
    });
    const int64_t patches = W->box_patches;
    // split the stack over gridDim.y only when the patches alone give less
    // than ~4 waves of 4 blocks per SM on 152 SMs
    const int64_t target_blocks = 152 * 4 * 4;
    int64_t chunks = (target_blocks + patches - 1) / patches;
    if (chunks < 1) chunks = 1;
    int64_t chunk = (stack + chunks - 1) / chunks;
    chunk = (chunk + SPS - 1) / SPS * SPS;
    if ((stack + chunk - 1) / chunk > 65535) chunk = ((stack + 65534) / 65535 + SPS - 1) / SPS * SPS;
    const int64_t nchunks = (stack + chunk - 1) / chunk;
    dim3 grid((unsigned)patches, (unsigned)nchunks);
    constexpr bool OUT64 = MODE != MODE_FAST;
    constexpr bool FF = MODE == MODE_FF;
    apply_patch_tma<SPS, NST, MINB, MODE, CT><<<grid, 32 * PATCH_WARPS, smem, s>>>(
        map, W->row_ptr, W->col, FF ? W->ff_slot : W->box_slot, FF ? W->ff_hi : W->box_val, FF ? W->ff_lo : nullptr,
        W->val32, W->val, OUT64 ? (double*)vout : nullptr, FastDiv((uint32_t)W->in_shape1), patch_grid(W), patches, W->box_origin, BR,
        stage_floats, box_bytes, vin, W->n_in, OUT64 ? nullptr : (float*)vout, W->n_out, stack, chunk, W->dflags,
        FF ? W->ff_perm : (OUT64 ? W->box_perm : nullptr));
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

// Tensor map of the input stack: columns x rows x slices, boxes of
// 32 columns x box_rows x bs slices, 128-byte swizzle.
bool encode_stack(const rg_weights_s* W, const float* vin, int64_t stack, int bs, CUtensorMap* map) {
    const cuuint64_t dims[3] = {(cuuint64_t)W->in_shape1, (cuuint64_t)W->in_shape0, (cuuint64_t)stack};
    const cuuint64_t strides[2] = {(cuuint64_t)W->in_shape1 * 4, (cuuint64_t)W->n_in * 4};
    const cuuint32_t box[3] = {(cuuint32_t)PBOX_C, (cuuint32_t)W->box_rows, (cuuint32_t)bs};
    const cuuint32_t estr[3] = {1, 1, 1};
    return encode_tiled()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)vin, dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int MODE>
int launch_box_config_mode(const rg_weights_s* W, int cfg, const float* vin, void* vout, int64_t stack,
                           cudaStream_t s) {
    const BoxConfig c = kBoxConfigs[cfg];
    // a stack shorter than a stage: the box carries only its slices (the
    // stage's other slices are never stored)
    const int bs = (int)std::min<int64_t>(c.sps, stack);
    CUtensorMap map;
    if (!encode_stack(W, vin, stack, MODE == MODE_FAST ? bs : 1, &map)) return RG_ERR_UNSUPPORTED;
    switch (cfg) {
        case 0: return launch_patch<4, 2, 0, MODE>(W, map, bs, vin, vout, stack, s);
        case 1: return launch_patch<4, 2, 4, MODE>(W, map, bs, vin, vout, stack, s);
        case 2: return launch_patch<4, 3, 4, MODE>(W, map, bs, vin, vout, stack, s);
        case 3: return launch_patch<2, 3, 4, MODE>(W, map, bs, vin, vout, stack, s);
        case 4: return launch_patch<2, 4, 4, MODE>(W, map, bs, vin, vout, stack, s);
        case 5: return launch_patch<8, 2, 0, MODE>(W, map, bs, vin, vout, stack, s);
        case 6: return launch_patch<4, 3, 0, MODE>(W, map, bs, vin, vout, stack, s);
    }
    return RG_ERR_UNSUPPORTED;
}

int launch_ff_config(const rg_weights_s* W, int cfg, const float* vin, void* vout, int64_t stack, cudaStream_t s) {
    const FFConfig c = kFFConfigs[cfg];
    const int bs = (int)std::min<int64_t>(c.sps, stack);
    CUtensorMap map;
    if (!encode_stack(W, vin, stack, 1, &map)) return RG_ERR_UNSUPPORTED;
    switch (cfg) {
        case 0: return launch_patch<6, 2, 0, MODE_FF, 6>(W, map, bs, vin, vout, stack, s);
        case 1: return launch_patch<8, 2, 0, MODE_FF, 6>(W, map, bs, vin, vout, stack, s);
        case 2: return launch_patch<4, 2, 0, MODE_FF, 6>(W, map, bs, vin, vout, stack, s);
        case 3: return launch_patch<4, 3, 0, MODE_FF, 6>(W, map, bs, vin, vout, stack, s);
        case 4: return launch_patch<2, 4, 0, MODE_FF, 6>(W, map, bs, vin, vout, stack, s);
        case 5: return launch_patch<4, 3, 3, MODE_FF, 4>(W, map, bs, vin, vout, stack, s);
        case 6: return launch_patch<4, 2, 4, MODE_FF, 0>(W, map, bs, vin, vout, stack, s);
    }
    return RG_ERR_UNSUPPORTED;
}

// MODE_FAST (float32 vout, kBoxConfigs) or MODE_FF (float64 vout, kFFConfigs).
int launch_box_config(const rg_weights_s* W, int mode, int cfg, const float* vin, void* vout, int64_t stack,
                      cudaStream_t s) {
    if (mode == MODE_FF) return launch_ff_config(W, cfg, vin, vout, stack, s);
    return launch_box_config_mode<MODE_FAST>(W, cfg, vin, vout, stack, s);
}

int forced_box_config(int mode) {
    if (mode == MODE_FF) {
        const char* env = getenv("RG_APPLY_FF_CONFIG");
        if (!env) return -1;
        int a = 0, b = 0, c = 0, d = 0;
        if (sscanf(env, "%d,%d,%d,%d", &a, &b, &c, &d) != 4) return -1;
        for (int k = 0; k < kNumFFConfigs; k++)
            if (kFFConfigs[k].sps == a && kFFConfigs[k].nst == b && kFFConfigs[k].minb == c &&
                kFFConfigs[k].cached == d)
                return k;
        return -1;
    }
    const char* env = getenv("RG_APPLY_BOX_CONFIG");
    if (!env) return -1;
    int a = 0, b = 0, c = 0;
    if (sscanf(env, "%d,%d,%d", &a, &b, &c) != 3) return -1;
    for (int k = 0; k < kNumBoxConfigs; k++)
        if (kBoxConfigs[k].sps == a && kBoxConfigs[k].nst == b && kBoxConfigs[k].minb == c) return k;
    return -1;
}

// Autotuner: on the first TMA apply of a handle in a stack size class, time
// every configuration on the real call (each run writes the same result) and
// keep the fastest for that class; later handles of the same kind (box
// height, stack size class) reuse the choice without timing.  The caller holds the handle's lock; synchronises
// the stream.
// Tuned configurations shared by handles of the same kind: box height and
// stack size class (1, 2-3, 4-7, ..., 64+) -> configuration.
std::mutex g_tuned_mutex;
std::map<std::tuple<int, int, int>, int> g_tuned;  // (mode, box rows, stack class) -> configuration

int tune_box(rg_weights_s* W, int mode, const float* vin, void* vout, int64_t stack, cudaStream_t s) {
    int& chosen = (mode == MODE_FF ? W->box_cfg_ff : W->box_cfg)[stack_class(stack)];
    if (chosen >= 0) return RG_OK;
    const int forced = forced_box_config(mode);
    if (forced >= 0) {
        chosen = forced;
        return RG_OK;
    }
    const std::tuple<int, int, int> kind(mode, W->box_rows, stack_class(stack));
    {
        std::lock_guard<std::mutex> lock(g_tuned_mutex);
        auto it = g_tuned.find(kind);
        if (it != g_tuned.end()) {
            chosen = it->second;
            return RG_OK;
        }
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    RG_CUDA(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaGetLastError();
        return RG_ERR_CUDA;
    }
    int best = -1;
    float best_ms = 0;
    int st = RG_OK;
    const int ncfg = mode == MODE_FF ? kNumFFConfigs : kNumBoxConfigs;
    for (int k = 0; k < ncfg && st == RG_OK; k++) {
        if (launch_box_config(W, mode, k, vin, vout, stack, s) != RG_OK) {  // warm-up; skips configs that do not fit
            cudaGetLastError();
            continue;
        }
        float ms = 0;
        for (int rep = 0; rep < 2; rep++) {
            cudaEventRecord(e0, s);
            launch_box_config(W, mode, k, vin, vout, stack, s);
            cudaEventRecord(e1, s);
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                set_error("apply (tuning): %s", cudaGetErrorString(cudaGetLastError()));
                st = RG_ERR_CUDA;
                break;
            }
            float tm = 0;
            cudaEventElapsedTime(&tm, e0, e1);
            ms = rep == 0 ? tm : std::min(ms, tm);
        }
        if (st == RG_OK && (best < 0 || ms < best_ms)) {
            best = k;
            best_ms = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != RG_OK) return st;
    chosen = best >= 0 ? best : -2;
    if (best >= 0) {
        std::lock_guard<std::mutex> lock(g_tuned_mutex);
        g_tuned[kind] = best;
    }
    return RG_OK;
}

// Launch the TMA apply; returns RG_ERR_UNSUPPORTED (nothing launched) when
// the tuned configuration does not take this call, so the caller can take
// another kernel.
int apply_box(const rg_weights_s* W, const float* vin, float* vout, int64_t stack, cudaStream_t s) {
    const int cfg = W->box_cfg[stack_class(stack)];
    if (cfg < 0) return RG_ERR_UNSUPPORTED;
    return launch_box_config(W, MODE_FAST, cfg, vin, vout, stack, s);
}

// The compensated (float-float) TMA apply with its tuned configuration.
int apply_box_ff(const rg_weights_s* W, const float* vin, double* vout, int64_t stack, cudaStream_t s) {
    const int cfg = W->box_cfg_ff[stack_class(stack)];
    if (W->box_state != 1 || cfg < 0 || !W->ff_slot || !W->ff_perm) return RG_ERR_UNSUPPORTED;
    return launch_box_config(W, MODE_FF, cfg, vin, vout, stack, s);
}

int tune_box_fast(rg_weights_s* W, const float* vin, float* vout, int64_t stack, cudaStream_t s) {
    return tune_box(W, MODE_FAST, vin, vout, stack, s);
}

int tune_box_ff(rg_weights_s* W, const float* vin, double* vout, int64_t stack, cudaStream_t s) {
    return tune_box(W, MODE_FF, vin, vout, stack, s);
}

// The exact (float64) TMA apply: 4 slices per stage, 2 stages (FP64 issue,
// not the staging, bounds it).
int apply_box_exact(const rg_weights_s* W, const float* vin, double* vout, int64_t stack, cudaStream_t s) {
    if (W->box_state != 1) return RG_ERR_UNSUPPORTED;
    const int bs = (int)std::min<int64_t>(4, stack);
    CUtensorMap map;
    if (!encode_stack(W, vin, stack, 1, &map)) return RG_ERR_UNSUPPORTED;
    return launch_patch<4, 2, 0, MODE_EXACT>(W, map, bs, vin, vout, stack, s);
}

// Whether the row kernel can take this call (the caller holds the lock and
// has made val32): a whole input slice fits a stage, every output fits a
// thread's registers, and the stack is long enough to fill the GPU.
// Builds the handle's row facts on first use (*made set).
int rows_usable(rg_weights_s* W, const float* vin, int64_t stack, cudaStream_t s, bool* made, bool* ok) {
    *ok = false;
    if (W->n_in % 4 != 0 || W->n_in > 12288 || W->n_out > (int64_t)ROWS_THREADS * ROWS_J || W->n_in >= INT32_MAX ||
        ((uintptr_t)vin & 15) != 0 || stack < 2 * 152)
        return RG_OK;
    if (W->rows_maxlen < 0) {
        unsigned* d = nullptr;
        RG_TRY(dalloc(&d, 1, s));
        cudaMemsetAsync(d, 0, sizeof(unsigned), s);
        max_row_len<<<grid_for(W->n_out, 256) > 1024 ? 1024 : grid_for(W->n_out, 256), 256, 0, s>>>(W->row_ptr,
                                                                                                   W->n_out, d);
        unsigned h = 0;
        small_to_host(&h, d, sizeof(unsigned), s);
        cudaError_t e = cudaStreamSynchronize(s);
        dfree(d, s);
        if (e != cudaSuccess) {
            set_error("apply (row facts): %s", cudaGetErrorString(e));
            return RG_ERR_CUDA;
        }
        W->rows_maxlen = (int)std::min<unsigned>(h, 1u << 30);
        if (W->dflags == nullptr) {
            RG_TRY(dalloc(&W->dflags, 1, s));
            cudaMemsetAsync(W->dflags, 0, sizeof(unsigned), s);
            *made = true;
        }
    }
    *ok = W->rows_maxlen <= ROWS_E;
    return RG_OK;
}

int apply_rows_launch(const rg_weights_s* W, const float* vin, float* vout, int64_t stack, cudaStream_t s) {
    const int stage_floats = (int)((W->n_in + 31) & ~31ll);  // stages start on 128-byte boundaries
    const size_t smem = (size_t)ROWS_NST * stage_floats * sizeof(float);
    static std::once_flag attr;
    std::call_once(attr, []() {
        cudaFuncSetAttribute(apply_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaGetLastError();
    });
    const int64_t blocks = std::min<int64_t>(stack, 152 * 2);
    apply_rows<<<(unsigned)blocks, ROWS_THREADS, smem, s>>>(W->row_ptr, W->col, W->val32, vin, W->n_in, vout,
                                                            W->n_out, stack, stage_floats, W->dflags);
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

}  // namespace rg
