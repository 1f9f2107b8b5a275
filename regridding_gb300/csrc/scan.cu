// Device-wide exclusive prefix sums (reduce-then-scan, three kernels).
#include "common.cuh"

namespace rg {
namespace {

constexpr int SCAN_BLOCK = 512;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

template <typename T>
__device__ __forceinline__ int64_t load_as_i64(const T* p, int64_t k, int64_t n) {
    return k < n ? (int64_t)p[k] : 0;
}

// inclusive block scan of one value per thread; returns the inclusive prefix
// and writes the block total to *total
__device__ int64_t block_inclusive_scan(int64_t v, int64_t* total) {
    __shared__ int64_t warp_sums[SCAN_BLOCK / 32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) warp_sums[warp] = v;
    __syncthreads();
    if (warp == 0) {
        int64_t w = lane < SCAN_BLOCK / 32 ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < SCAN_BLOCK / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    if (warp > 0) v += warp_sums[warp - 1];
    *total = warp_sums[SCAN_BLOCK / 32 - 1];
    __syncthreads();
    return v;
}

template <typename T>
__global__ void __launch_bounds__(SCAN_BLOCK) tile_sums(const T* in, int64_t n, int64_t* sums) {
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) s += load_as_i64(in, base + k, n);
    int64_t total;
    block_inclusive_scan(s, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

template <typename T>
__global__ void __launch_bounds__(SCAN_BLOCK)
    tile_scan(const T* in, int64_t* out, int64_t n, const int64_t* tile_offsets, int64_t* total_dev) {
    int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
    int64_t v[SCAN_ITEMS];
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        v[k] = load_as_i64(in, base + k, n);
        s += v[k];
    }
    int64_t total;
    int64_t incl = block_inclusive_scan(s, &total);
    int64_t run = incl - s + (tile_offsets ? tile_offsets[blockIdx.x] : 0);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (total_dev && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
        *total_dev = (tile_offsets ? tile_offsets[blockIdx.x] : 0) + total;
    }
}

template <typename T>
int scan_impl(const T* in, int64_t* out, int64_t n, int64_t* total_dev, cudaStream_t s) {
    if (n <= 0) {
        if (total_dev) RG_TRY(zero_async(total_dev, sizeof(int64_t), s));
        return RG_OK;
    }
    int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles == 1) {
        tile_scan<T><<<1, SCAN_BLOCK, 0, s>>>(in, out, n, nullptr, total_dev);
        RG_CUDA(cudaGetLastError());
        return RG_OK;
    }
    int64_t* sums = nullptr;
    RG_TRY(dalloc(&sums, (size_t)tiles, s));
    tile_sums<T><<<(unsigned)tiles, SCAN_BLOCK, 0, s>>>(in, n, sums);
    int st = RG_OK;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("tile_sums: %s", cudaGetErrorString(e));
        st = RG_ERR_CUDA;
    }
    if (st == RG_OK) st = scan_impl<int64_t>(sums, sums, tiles, nullptr, s);
    if (st == RG_OK) {
        tile_scan<T><<<(unsigned)tiles, SCAN_BLOCK, 0, s>>>(in, out, n, sums, total_dev);
        e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error("tile_scan: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
        }
    }
    dfree(sums, s);
    return st;
}

}  // namespace

int exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n, int64_t* total_dev,
                       cudaStream_t s) {
    return scan_impl<int64_t>(in, out, n, total_dev, s);
}

int exclusive_scan_u32_to_i64(const unsigned* in, int64_t* out, int64_t n, int64_t* total_dev,
                              cudaStream_t s) {
    return scan_impl<unsigned>(in, out, n, total_dev, s);
}

}  // namespace rg
