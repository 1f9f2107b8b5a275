// Bucketed stable ordering: counting sort on a primary bucket key followed by
// an in-bucket ranking on a unique secondary key.  This is how raw sweep
// triples are grouped by output cell (and entries by input cell for the
// transposed layouts) without a full-width radix sort: buckets are short
// (tens of entries), so ranking inside each bucket is cheap and exact.
#include "common.cuh"

namespace rg {
namespace {

constexpr int SMALL_BUCKET = 64;  // ranked by one thread per element
constexpr int RANK_TILE = 2048;   // keys staged per shared-memory tile for long buckets

// Consecutive elements often share a bucket (a sweep emits the entries of a
// cell together): the lanes of a warp with the same bucket add to its counter
// once.  The loops run whole warps (uniform trip counts) for the collectives.
__device__ __forceinline__ unsigned warp_bucket_add(unsigned* counters, int32_t b, bool active) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned key = active ? (unsigned)b : 0xffffffffu;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const unsigned leader = __ffs(peers) - 1;
    unsigned base = 0;
    if (active && lane == leader) base = atomicAdd(&counters[b], (unsigned)__popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + __popc(peers & ((1u << lane) - 1u));
}

__global__ void count_buckets(const int32_t* bucket, int64_t n, unsigned* counts) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k0 = blockIdx.x * (int64_t)blockDim.x; k0 < n; k0 += stride) {
        const int64_t k = k0 + threadIdx.x;
        const bool active = k < n;
        (void)warp_bucket_add(counts, active ? bucket[k] : 0, active);
    }
}

__global__ void scatter_buckets(const int32_t* bucket, const int64_t* skey, int64_t n,
                                const int64_t* bucket_ptr, unsigned* cursor, uint32_t* tmp_idx,
                                int64_t* tmp_key) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k0 = blockIdx.x * (int64_t)blockDim.x; k0 < n; k0 += stride) {
        const int64_t k = k0 + threadIdx.x;
        const bool active = k < n;
        const int32_t b = active ? bucket[k] : 0;
        const unsigned pos = warp_bucket_add(cursor, b, active);
        if (active) {
            const int64_t dst = bucket_ptr[b] + pos;
            tmp_idx[dst] = (uint32_t)k;
            tmp_key[dst] = skey[k];
        }
    }
}

// One thread per element of a short bucket: its rank is the number of keys in
// the bucket smaller than its own.  Elements of long buckets are skipped and
// their buckets listed (once, by the bucket's first element) for rank_long.
__global__ void rank_small(const int32_t* bucket, const uint32_t* tmp_idx, const int64_t* tmp_key,
                           int64_t n, const int64_t* bucket_ptr, uint32_t* perm, int32_t* long_list,
                           unsigned* long_count, const double* val, int32_t* out_hi, double* out_val) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
        uint32_t idx = tmp_idx[e];
        int32_t b = bucket[idx];
        int64_t s = bucket_ptr[b], t = bucket_ptr[b + 1];
        if (t - s > SMALL_BUCKET) {
            if (e == s) long_list[atomicAdd(long_count, 1u)] = b;
            continue;
        }
        int64_t key = tmp_key[e];
        int64_t rank = 0;
        for (int64_t q = s; q < t; q++) rank += tmp_key[q] < key;
        perm[s + rank] = idx;
        if (out_val) {
            out_hi[s + rank] = (int32_t)(key >> 32);
            out_val[s + rank] = val[idx];
        }
    }
}

// One block per long bucket (grid-stride over the list built by rank_small).
__global__ void __launch_bounds__(256)
    rank_long(const uint32_t* tmp_idx, const int64_t* tmp_key, const int64_t* bucket_ptr,
              const int32_t* long_list, const unsigned* long_count, uint32_t* perm, const double* val,
              int32_t* out_hi, double* out_val) {
    __shared__ int64_t tile[RANK_TILE];
    unsigned nl = *long_count;
    for (unsigned li = blockIdx.x; li < nl; li += gridDim.x) {
        int32_t b = long_list[li];
        int64_t s = bucket_ptr[b], t = bucket_ptr[b + 1];
        int64_t len = t - s;
        // each thread owns elements e = s + threadIdx.x + r * blockDim.x
        for (int64_t e0 = s; e0 < t; e0 += (int64_t)blockDim.x * 8) {
            int64_t mykey[8];
            int64_t rank[8];
#pragma unroll
            for (int r = 0; r < 8; r++) {
                int64_t e = e0 + threadIdx.x + (int64_t)r * blockDim.x;
                mykey[r] = e < t ? tmp_key[e] : INT64_MAX;
                rank[r] = 0;
            }
            for (int64_t q0 = 0; q0 < len; q0 += RANK_TILE) {
                int64_t m = len - q0 < RANK_TILE ? len - q0 : RANK_TILE;
                __syncthreads();
                for (int64_t q = threadIdx.x; q < m; q += blockDim.x) tile[q] = tmp_key[s + q0 + q];
                __syncthreads();
                for (int64_t q = 0; q < m; q++) {
                    int64_t kq = tile[q];
#pragma unroll
                    for (int r = 0; r < 8; r++) rank[r] += kq < mykey[r];
                }
            }
#pragma unroll
            for (int r = 0; r < 8; r++) {
                int64_t e = e0 + threadIdx.x + (int64_t)r * blockDim.x;
                if (e < t) {
                    const uint32_t idx = tmp_idx[e];
                    perm[s + rank[r]] = idx;
                    if (out_val) {
                        out_hi[s + rank[r]] = (int32_t)(mykey[r] >> 32);
                        out_val[s + rank[r]] = val[idx];
                    }
                }
            }
        }
        __syncthreads();
    }
}

}  // namespace

int bucket_sort(const int32_t* bucket, const int64_t* skey, int64_t n, int64_t nbuckets,
                int64_t* bucket_ptr, uint32_t* perm, unsigned* flags, cudaStream_t s, const double* val,
                int32_t* out_hi, double* out_val) {
    if (!(val && out_hi && out_val)) val = nullptr, out_hi = nullptr, out_val = nullptr;
    (void)flags;
    RG_CHECK(n < (int64_t)UINT32_MAX, RG_ERR_UNSUPPORTED,
             "bucket_sort: %lld elements exceed the 32-bit index range", (long long)n);
    unsigned *counts = nullptr, *long_count = nullptr;
    uint32_t* tmp_idx = nullptr;
    int64_t* tmp_key = nullptr;
    int32_t* long_list = nullptr;
    int st = RG_OK;
    do {
        if ((st = dalloc(&counts, (size_t)nbuckets + 1, s))) break;
        if ((st = dalloc(&long_count, 1, s))) break;
        if ((st = dalloc(&tmp_idx, (size_t)n, s))) break;
        if ((st = dalloc(&tmp_key, (size_t)n, s))) break;
        if ((st = dalloc(&long_list, (size_t)nbuckets, s))) break;
        zero_async(counts, sizeof(unsigned) * (nbuckets + 1), s);
        zero_async(long_count, sizeof(unsigned), s);
        if (n > 0) count_buckets<<<grid_for(n, 256) > 4096 ? 4096 : grid_for(n, 256), 256, 0, s>>>(
            bucket, n, counts);
        if ((st = exclusive_scan_u32_to_i64(counts, bucket_ptr, nbuckets + 1, nullptr, s))) break;
        zero_async(counts, sizeof(unsigned) * (nbuckets + 1), s);
        if (n > 0) {
            unsigned g = grid_for(n, 256) > 8192 ? 8192 : grid_for(n, 256);
            scatter_buckets<<<g, 256, 0, s>>>(bucket, skey, n, bucket_ptr, counts, tmp_idx, tmp_key);
            rank_small<<<g, 256, 0, s>>>(bucket, tmp_idx, tmp_key, n, bucket_ptr, perm, long_list,
                                         long_count, val, out_hi, out_val);
            rank_long<<<1024, 256, 0, s>>>(tmp_idx, tmp_key, bucket_ptr, long_list, long_count, perm, val, out_hi,
                                           out_val);
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error("bucket_sort: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
        }
    } while (0);
    dfree(counts, s);
    dfree(long_count, s);
    dfree(tmp_idx, s);
    dfree(tmp_key, s);
    dfree(long_list, s);
    return st;
}

}  // namespace rg
