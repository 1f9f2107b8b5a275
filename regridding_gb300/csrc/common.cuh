// Shared helpers for the regridding_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <mutex>
#include <string>

#include <nvtx3/nvToolsExt.h>

#include "../../include/regrid_gb300.h"

namespace rg {

// A named NVTX range over the extent of a C entry point, shown by the Nsight
// tools on the host timeline (without a tool attached a push or pop is a
// check of an unset function pointer).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// ---------------------------------------------------------------------------
// error reporting: every C entry point returns an RG_* status and records a
// message retrievable through rg_last_error (thread-local).
// ---------------------------------------------------------------------------
void set_error(const char* fmt, ...);
const char* last_error();

#define RG_CUDA(call)                                                                  \
    do {                                                                               \
        cudaError_t _e = (call);                                                       \
        if (_e != cudaSuccess) {                                                       \
            ::rg::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call,                 \
                            cudaGetErrorString(_e));                                   \
            return RG_ERR_CUDA;                                                        \
        }                                                                              \
    } while (0)

#define RG_CHECK(cond, status, ...)                                                    \
    do {                                                                               \
        if (!(cond)) {                                                                 \
            ::rg::set_error(__VA_ARGS__);                                              \
            return (status);                                                           \
        }                                                                              \
    } while (0)

#define RG_TRY(expr)                                                                   \
    do {                                                                               \
        int _s = (expr);                                                               \
        if (_s != RG_OK) return _s;                                                    \
    } while (0)

// Device-side error flag bits, written with atomicOr by kernels that detect a
// condition they cannot handle (a walk exceeding its step cap, a seat outside
// the grid, an over-long bucket).  The host reads the word after the launch
// sequence and turns it into a status.
enum DeviceFlag : unsigned {
    FLAG_WALK_CAP = 1u << 0,
    FLAG_SEAT_OUTSIDE = 1u << 1,
    FLAG_BUCKET_TOO_LONG = 1u << 2,
    FLAG_CAPACITY = 1u << 3,
    FLAG_TIMEOUT = 1u << 4,  // a bounded wait for an asynchronous copy gave up
    FLAG_BOUNDS = 1u << 5,   // (debug builds, -DRG_DEBUG) a grid read outside its array
};

// ---------------------------------------------------------------------------
// IEEE double arithmetic with one rounding per operation.  The upstream
// algorithms are defined by their (unfused) Python arithmetic, so every FP64
// expression whose result decides a branch or is emitted as a weight is spelt
// with these intrinsics, which the compiler never contracts into an FMA.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// float32 -> float64, exactly, with integer operations only (the FP64 pipe
// of a GB300 issues 2 operations per clock per SM and is kept for the sums):
// a normal binary32 value keeps its sign, its exponent is rebiased from 127
// to 1023 and its 23 fraction bits are followed by 29 zeros; a subnormal
// man * 2^-149 is normalised at its leading bit; zeros keep their sign;
// infinities and NaNs keep their payload under the all-ones exponent.
__device__ __forceinline__ double widen(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned ex = (u >> 23) & 0xffu, man = u & 0x7fffffu;
    unsigned long long e64 = 0ull, m64 = 0ull;
    if (ex != 0u) {
        e64 = ex == 0xffu ? 0x7ffull : (unsigned long long)(ex + (1023u - 127u));
        m64 = (unsigned long long)man << 29;
    } else if (man != 0u) {
        const int lead = 31 - __clz((int)man);  // 0..22
        e64 = (unsigned long long)(lead + 1023 - 149);
        m64 = ((unsigned long long)man << (52 - lead)) & 0xfffffffffffffull;
    }
    return __longlong_as_double((long long)(((unsigned long long)(u >> 31) << 63) | (e64 << 52) | m64));
}

constexpr int64_t MAXSIZE = INT64_MAX;  // sys.maxsize: the upstream out-of-grid sentinel

// Keep up to this many bytes of freed stream-ordered memory in the current
// device's default pool instead of returning it to the driver at every
// synchronisation (the pool is this process's; the setting ends with it).
// Builds allocate and free their scratch every call; without it each build
// maps its scratch anew.  RG_POOL_KEEP_BYTES overrides.  Implemented in
// capi.cu; once per device.
constexpr uint64_t POOL_KEEP_BYTES = 32ull << 30;
void init_pool_once();

// simple RAII-free device buffer helpers (stream ordered)
template <typename T>
int dalloc(T** p, size_t n, cudaStream_t s) {
    *p = nullptr;
    init_pool_once();
    if (n == 0) n = 1;
    cudaError_t e = cudaMallocAsync((void**)p, n * sizeof(T), s);
    if (e != cudaSuccess) {
        cudaGetLastError();  // a failed allocation must not leave a sticky error for later checks
        set_error("cudaMallocAsync(%zu bytes): %s", n * sizeof(T), cudaGetErrorString(e));
        return RG_ERR_ALLOC;
    }
    return RG_OK;
}
template <typename T>
void dfree(T* p, cudaStream_t s) {
    if (p) cudaFreeAsync((void*)p, s);
}

// Unsigned 32-bit division by a divisor fixed for a launch, as a multiply
// and two shifts (Granlund and Montgomery, "Division by invariant integers
// using multiplication", PLDI 1994, figure 4.1): exact for every dividend
// and every divisor 1 <= d < 2^31, and it keeps the division's reciprocal
// and correction sequence off the kernel's critical path.
struct FastDiv {
    uint32_t d, m, s1, s2;
    FastDiv() = default;
    explicit FastDiv(uint32_t div) : d(div) {
        uint32_t l = 0;
        while (l < 32 && (1ull << l) < div) ++l;  // ceil(log2 d)
        m = (uint32_t)((((1ull << 32) * ((1ull << l) - div)) / div) + 1);
        s1 = l < 1 ? l : 1;
        s2 = l > 1 ? l - 1 : 0;
    }
    __device__ __forceinline__ uint32_t div(uint32_t n) const {
        const uint32_t t1 = __umulhi(m, n);
        return (t1 + ((n - t1) >> s1)) >> s2;
    }
};

// Small host <-> device transfers (sizes, flags, per-pair parameters).  On a
// device whose kernels read and write pageable host memory (the Grace host
// of a GB300: address translation over NVLink-C2C) a small kernel moves
// them, so they do not queue on the copy engines behind other streams' large
// transfers (a 512^2 build took 6-9 ms instead of 1.3 ms next to a stream
// copying 600 MB blocks); elsewhere cudaMemcpyAsync.  small_to_host is
// stream-ordered: read the destination after synchronising the stream.
// small_to_device returns once the source has been read (it synchronises the
// stream when a kernel did the copy), so the source may be freed at once.
bool kernel_host_access();
// cudaMemsetAsync(p, 0, n, s) as a kernel, for the small clears of the build
int zero_async(void* p, size_t n, cudaStream_t s);
int small_to_host(void* h_dst, const void* d_src, size_t n, cudaStream_t s);
int small_to_device(void* d_dst, const void* h_src, size_t n, cudaStream_t s);

inline unsigned grid_for(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 0x7fffffff) g = 0x7fffffff;
    return (unsigned)g;
}

// device-wide exclusive scan of n int64 values (in may equal out); writes the
// total to *total_dev if non-null.  Implemented in scan.cu.
int exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n, int64_t* total_dev,
                       cudaStream_t s);
int exclusive_scan_u32_to_i64(const unsigned* in, int64_t* out, int64_t n, int64_t* total_dev,
                              cudaStream_t s);

// Stable ordering of elements grouped into buckets: given bucket[k] in
// [0, nbuckets) and a secondary key skey[k] that is unique within each bucket,
// produce bucket_ptr[nbuckets+1] and perm[n] such that perm lists the
// elements sorted by (bucket, skey).  With a payload (val[k], and out_hi /
// out_val non-null) the sorted high halves of the keys and the values are
// written in the same order (out_hi[g] = skey[perm[g]] >> 32, out_val[g] =
// val[perm[g]]), gathered while ranking.  Implemented in sort.cu.
int bucket_sort(const int32_t* bucket, const int64_t* skey, int64_t n, int64_t nbuckets,
                int64_t* bucket_ptr, uint32_t* perm, unsigned* flags, cudaStream_t s,
                const double* val = nullptr, int32_t* out_hi = nullptr, double* out_val = nullptr);

// Stack size classes of the apply autotuner (1, 2-3, 4-7, ..., 32-63, 64 and
// more slices).  A handle keeps one tuned configuration per class: the best
// number of slices per stage depends on how many slices a call has (a stage
// computes all its slices, also those past the end of the stack).
constexpr int kStackClasses = 7;
inline int stack_class(int64_t stack) {
    int c = 0;
    while (c < kStackClasses - 1 && ((int64_t)2 << c) <= stack) c++;
    return c;
}

}  // namespace rg

// Opaque weight matrix of one orthogonal element, resident on the device.
// Rows are output cells, columns input cells; entries of each row are sorted
// by column, which is also the order the upstream apply accumulates them.
struct rg_weights_s {
    int64_t n_in = 0, n_out = 0, nnz = 0;
    int64_t* row_ptr = nullptr;  // [n_out + 1]
    int32_t* col = nullptr;      // [nnz]
    double* val = nullptr;       // [nnz]
    float* val32 = nullptr;      // lazily made float32 copy of val
    // transposed (rows = input cells), built on demand for the transposed apply
    int64_t* t_row_ptr = nullptr;
    int32_t* t_col = nullptr;
    double* t_val = nullptr;
    float* t_val32 = nullptr;
    // (optional) output grid shape for 2D tiling of the apply, and input grid
    // shape for the tensor-map (TMA) staging of the input slices
    int64_t out_shape0 = 0, out_shape1 = 0;
    int64_t in_shape0 = 0, in_shape1 = 0;
    // warp-tile lists of the float32 fast apply, built on first use; index 0
    // lists single cells, index 1 lists 32-byte sectors of 8 cells
    bool tiled_ready[2] = {false, false};
    int64_t t_tiles = 0;
    int t_gmax[2] = {0, 0};
    int64_t* t_gptr[2] = {nullptr, nullptr};   // [tiles + 1]
    int32_t* t_gidx[2] = {nullptr, nullptr};   // the lists
    uint16_t* t_slot[2] = {nullptr, nullptr};  // [nnz] staged slot of each entry
    // patch lists of the TMA apply: per 16 x 16 patch of output cells the
    // origin (row, column) of a fixed box_rows x box_cols box of input cells
    // holding its footprint (row -1: no entries, -2: footprint larger than
    // the box), and per entry its (swizzled) offset in the box
    int box_state = 0;  // 0 not built, 1 ready, -1 not applicable
    int box_rows = 0, box_cols = 0;
    int64_t box_patches = 0;
    // configuration chosen by the autotuner per stack class (-1 not tuned, -2 none fits)
    int box_cfg[rg::kStackClasses] = {-1, -1, -1, -1, -1, -1, -1};
    int2* box_origin = nullptr;
    uint16_t* box_slot = nullptr;  // per entry, in the order the TMA kernel gathers them
    uint8_t* box_perm = nullptr;   // exact apply: per patch, thread -> output (longest rows first)
    float* box_val = nullptr;      // float32 weights in that order
    // the compensated (float-float) apply: per entry its box slot, float32
    // weight hi = (float)w and rest lo = (float)(w - hi), in the order its
    // row-length thread layout (ff_perm) gathers them; its tuned configuration
    uint8_t* ff_perm = nullptr;    // compensated apply: per patch, thread -> output (row-length classes)
    uint16_t* ff_slot = nullptr;
    float* ff_hi = nullptr;
    float* ff_lo = nullptr;
    int box_cfg_ff[rg::kStackClasses] = {-1, -1, -1, -1, -1, -1, -1};
    unsigned* dflags = nullptr;  // device error word of the asynchronous (TMA) apply
    int rows_maxlen = -1;        // longest row (for the row kernel; -1 not known yet)
    int device = 0;
    std::mutex mu;  // guards the lazily made state above (made on first use by an apply)
};

namespace rg {

// One grid pair of a conservative build (device pointers; row-major vertex
// arrays of nx x ny; w_in nullable).
struct PairSpec {
    const double *xi, *yi;
    int64_t nxi, nyi;
    const double *xo, *yo;
    int64_t nxo, nyo;
    const double* w_in;
};

// Conservative weights of G pairs in one pass (conservative2d.cu); W[g] are
// empty handles that receive the CSR of pair g when status[g] is RG_OK.
int build_batch(const PairSpec* pairs, int G, cudaStream_t s, rg_weights_s** W, int* status);

}  // namespace rg

