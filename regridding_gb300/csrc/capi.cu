// extern "C" entry points of libregrid_gb300 (declared in include/regrid_gb300.h).
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "common.cuh"

namespace rg {

static thread_local char g_err[1024] = {0};

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}
const char* last_error() { return g_err; }

// implemented in the kernel files
int build_conservative_2d(const double*, const double*, int64_t, int64_t, const double*, const double*,
                          int64_t, int64_t, const double*, cudaStream_t, rg_weights_s*);
int cell_area_2d(const double*, const double*, int64_t, int64_t, double*, cudaStream_t);
int locate_2d_exact(const double*, const double*, int64_t, int64_t, const double*, const double*, int64_t,
                    int, int64_t*, int64_t*, cudaStream_t);
int locate_2d_walk(const double*, const double*, int64_t, int64_t, const double*, const double*, int64_t,
                   int64_t*, int64_t*, cudaStream_t);
int apply_weights(rg_weights_s*, bool, const void*, int, void*, int, int64_t, int, cudaStream_t);
int apply_host(rg_weights_s*, const void*, int, void*, int, int64_t, int, int64_t, cudaStream_t);
int find_indices_1d(const double*, int64_t, int64_t, const double*, int64_t, int64_t, int64_t, int, int64_t,
                    int64_t*, cudaStream_t);
int multilinear_1d(const double*, int64_t, int64_t, const double*, const double*, int64_t, int64_t, int64_t,
                   const double*, int64_t, int, int64_t*, int64_t*, double*, int64_t*, cudaStream_t);
int conservative_1d(const double*, int64_t, int64_t, const double*, int64_t, int64_t, int64_t, const double*,
                    int64_t, int64_t, int64_t*, int64_t*, double*, int64_t*, cudaStream_t);
int cell_length_1d(const double*, int64_t, int64_t, double*, cudaStream_t);
int transpose_conservative_scale(const int64_t*, const int64_t*, const double*, int64_t, const double*,
                                 int64_t, const double*, int64_t, const double*, double*, cudaStream_t);

namespace {

// entries of a COO list normalised to [0, n) (numpy-style negative indices)
__global__ void normalise_coo(const int64_t* in, const int64_t* out, int64_t nnz, int64_t n_in,
                              int64_t n_out, int32_t* in32, int32_t* out32, int64_t* pos,
                              unsigned* bad) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz;
         k += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = in[k], o = out[k];
        if (i < 0) i += n_in;
        if (o < 0) o += n_out;
        if (i < 0 || i >= n_in || o < 0 || o >= n_out) {
            atomicOr(bad, 1u);
            i = 0;
            o = 0;
        }
        in32[k] = (int32_t)i;
        out32[k] = (int32_t)o;
        pos[k] = k;
    }
}

__global__ void gather_csr(const uint32_t* perm, const int32_t* in32, const double* val, int64_t nnz,
                           int32_t* col, double* cval) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz;
         k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t e = perm[k];
        col[k] = in32[e];
        cval[k] = val[e];
    }
}

// row index of every stored entry, and the key (row, position) that orders
// entries of equal column by row
__global__ void expand_rows(const int64_t* row_ptr, int64_t n_rows, int32_t* row_of, int64_t* key) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_rows;
         r += (int64_t)gridDim.x * blockDim.x) {
        for (int64_t k = row_ptr[r]; k < row_ptr[r + 1]; k++) {
            row_of[k] = (int32_t)r;
            key[k] = ((int64_t)r << 32) | (int64_t)(uint32_t)k;
        }
    }
}

__global__ void gather_transposed(const uint32_t* perm, const int32_t* row_of, const double* val,
                                  int64_t nnz, int32_t* t_col, double* t_val) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz;
         k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t e = perm[k];
        t_col[k] = row_of[e];
        t_val[k] = val[e];
    }
}

__global__ void gather_export(const uint32_t* perm, const int32_t* col, const int32_t* row_of,
                              const double* val, int64_t nnz, int64_t* e_in, int64_t* e_out,
                              double* e_val) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz;
         k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t e = perm[k];
        e_in[k] = col[e];
        e_out[k] = row_of[e];
        e_val[k] = val[e];
    }
}

inline unsigned capped(int64_t n, int block, unsigned cap = 65536) {
    unsigned g = grid_for(n, block);
    return g > cap ? cap : g;
}

// Column-major order of the stored entries: perm over CSR positions sorted
// by (column, row), plus the row of every entry.
int column_order(rg_weights_s* W, int32_t** row_of, uint32_t** perm, int64_t** col_ptr,
                 cudaStream_t s) {
    int64_t* key = nullptr;
    int st = RG_OK;
    *row_of = nullptr;
    *perm = nullptr;
    *col_ptr = nullptr;
    do {
        if ((st = dalloc(row_of, (size_t)W->nnz, s))) break;
        if ((st = dalloc(&key, (size_t)W->nnz, s))) break;
        if ((st = dalloc(perm, (size_t)W->nnz, s))) break;
        if ((st = dalloc(col_ptr, (size_t)W->n_in + 1, s))) break;
        expand_rows<<<capped(W->n_out, 128), 128, 0, s>>>(W->row_ptr, W->n_out, *row_of, key);
        st = bucket_sort(W->col, key, W->nnz, W->n_in, *col_ptr, *perm, nullptr, s);
    } while (0);
    dfree(key, s);
    if (st) {
        dfree(*row_of, s);
        dfree(*perm, s);
        dfree(*col_ptr, s);
        *row_of = nullptr;
        *perm = nullptr;
        *col_ptr = nullptr;
    }
    return st;
}

void free_weights(rg_weights_s* W, cudaStream_t s) {
    dfree(W->row_ptr, s);
    dfree(W->col, s);
    dfree(W->val, s);
    dfree(W->val32, s);
    dfree(W->t_row_ptr, s);
    dfree(W->t_col, s);
    dfree(W->t_val, s);
    dfree(W->t_val32, s);
    for (int g = 0; g < 2; g++) {
        dfree(W->t_gptr[g], s);
        dfree(W->t_gidx[g], s);
        dfree(W->t_slot[g], s);
    }
    dfree(W->box_origin, s);
    dfree(W->box_slot, s);
    dfree(W->box_val, s);
    dfree(W->ff_slot, s);
    dfree(W->ff_hi, s);
    dfree(W->ff_lo, s);
    dfree(W->box_perm, s);
    dfree(W->ff_perm, s);
    dfree(W->dflags, s);
    delete W;
}

}  // namespace

void init_pool_once() {
    static std::once_flag flags[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return;
    }
    std::call_once(flags[dev], [dev]() {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t keep = POOL_KEEP_BYTES;
            if (const char* env = getenv("RG_POOL_KEEP_BYTES")) keep = strtoull(env, nullptr, 10);
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        cudaGetLastError();
    });
}

// Build the CSC (rows = input cells) for the transposed apply; the caller
// holds the handle's lock.
int ensure_transposed(rg_weights_s* W, cudaStream_t s) {
    if (W->t_row_ptr) return RG_OK;
    int32_t* row_of = nullptr;
    uint32_t* perm = nullptr;
    int64_t* col_ptr = nullptr;
    RG_TRY(column_order(W, &row_of, &perm, &col_ptr, s));
    int st = RG_OK;
    do {
        if ((st = dalloc(&W->t_col, (size_t)W->nnz, s))) break;
        if ((st = dalloc(&W->t_val, (size_t)W->nnz, s))) break;
        if (W->nnz > 0)
            gather_transposed<<<capped(W->nnz, 256), 256, 0, s>>>(perm, row_of, W->val, W->nnz, W->t_col,
                                                                 W->t_val);
        W->t_row_ptr = col_ptr;
        col_ptr = nullptr;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error("transpose: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
        }
    } while (0);
    dfree(row_of, s);
    dfree(perm, s);
    dfree(col_ptr, s);
    return st;
}

namespace {

__global__ void host_bytes_copy(unsigned char* __restrict__ dst, const unsigned char* __restrict__ src, size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if ((((uintptr_t)dst | (uintptr_t)src | n) & 7) == 0) {
        unsigned long long* d8 = (unsigned long long*)dst;
        const unsigned long long* s8 = (const unsigned long long*)src;
        for (size_t k = t0; k < n / 8; k += stride) d8[k] = s8[k];
    } else {
        for (size_t k = t0; k < n; k += stride) dst[k] = src[k];
    }
}

__global__ void zero_bytes(unsigned char* __restrict__ p, size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if ((((uintptr_t)p | n) & 7) == 0) {
        unsigned long long* p8 = (unsigned long long*)p;
        for (size_t k = t0; k < n / 8; k += stride) p8[k] = 0ull;
    } else {
        for (size_t k = t0; k < n; k += stride) p[k] = 0;
    }
}

constexpr int kMaxDevices = 64;
int g_host_access[kMaxDevices];  // per device ordinal: 0 not queried yet, 1 yes, 2 no
std::mutex g_host_access_mu;

}  // namespace

// Whether kernels on the CURRENT device may dereference pageable host
// pointers (queried once per device ordinal: devices of one process can
// differ).
bool kernel_host_access() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return false;
    }
    std::lock_guard<std::mutex> lock(g_host_access_mu);
    if (g_host_access[dev] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
            cudaGetLastError();
            v = 0;
        }
        g_host_access[dev] = v ? 1 : 2;
    }
    return g_host_access[dev] == 1;
}

static unsigned small_blocks(size_t n) {
    // one 8-byte word per thread and pass; 256 blocks read a pageable host
    // array at ~170-190 GB/s on GB300 (64: ~130-140), more add nothing
    const size_t b = (n / 8 + 255) / 256;
    return (unsigned)(b < 1 ? 1 : (b > 256 ? 256 : b));
}

int zero_async(void* p, size_t n, cudaStream_t s) {
    if (n == 0) return RG_OK;
    const size_t b = (n / 8 + 255) / 256;
    zero_bytes<<<(unsigned)(b < 1 ? 1 : (b > 1024 ? 1024 : b)), 256, 0, s>>>((unsigned char*)p, n);
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

int small_to_host(void* h_dst, const void* d_src, size_t n, cudaStream_t s) {
    if (n == 0) return RG_OK;
    if (!kernel_host_access()) {
        RG_CUDA(cudaMemcpyAsync(h_dst, d_src, n, cudaMemcpyDeviceToHost, s));
        return RG_OK;
    }
    host_bytes_copy<<<small_blocks(n), 256, 0, s>>>((unsigned char*)h_dst, (const unsigned char*)d_src, n);
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

int small_to_device(void* d_dst, const void* h_src, size_t n, cudaStream_t s) {
    if (n == 0) return RG_OK;
    if (!kernel_host_access()) {
        RG_CUDA(cudaMemcpyAsync(d_dst, h_src, n, cudaMemcpyHostToDevice, s));
        return RG_OK;
    }
    host_bytes_copy<<<small_blocks(n), 256, 0, s>>>((unsigned char*)d_dst, (const unsigned char*)h_src, n);
    RG_CUDA(cudaGetLastError());
    RG_CUDA(cudaStreamSynchronize(s));
    return RG_OK;
}

}  // namespace rg

using namespace rg;

extern "C" {

int rg_version(void) { return 200; }

int rg_copy_from_host(void* d_dst, const void* h_src, int64_t nbytes, rg_stream_t stream) {
    RG_CHECK(nbytes >= 0 && (nbytes == 0 || (d_dst && h_src)), RG_ERR_ARG, "rg_copy_from_host: bad arguments");
    return small_to_device(d_dst, h_src, (size_t)nbytes, (cudaStream_t)stream);
}

int rg_device_attributes(int64_t* h_out, int n) {
    RG_CHECK(h_out && n >= 0, RG_ERR_ARG, "rg_device_attributes: NULL output");
    int dev = 0;
    RG_CUDA(cudaGetDevice(&dev));
    const cudaDeviceAttr attrs[] = {cudaDevAttrMultiProcessorCount, cudaDevAttrAsyncEngineCount,
                                    cudaDevAttrPageableMemoryAccess,
                                    cudaDevAttrPageableMemoryAccessUsesHostPageTables,
                                    cudaDevAttrCanUseHostPointerForRegisteredMem, cudaDevAttrConcurrentManagedAccess};
    const int na = (int)(sizeof(attrs) / sizeof(attrs[0]));
    for (int k = 0; k < n && k < na; ++k) {
        int v = 0;
        RG_CUDA(cudaDeviceGetAttribute(&v, attrs[k], dev));
        h_out[k] = v;
    }
    return RG_OK;
}

int rg_last_error(char* buf, size_t n) {
    size_t len = strlen(g_err);
    if (buf && n) {
        size_t c = len < n - 1 ? len : n - 1;
        memcpy(buf, g_err, c);
        buf[c] = 0;
    }
    return (int)len;
}

int rg_build_conservative_2d(const double* d_xi, const double* d_yi, int64_t nxi, int64_t nyi,
                             const double* d_xo, const double* d_yo, int64_t nxo, int64_t nyo,
                             const double* d_w_in, rg_stream_t stream, rg_weights* out) {
    rg::NvtxRange nvtx_range("rg_build_conservative_2d");
    RG_CHECK(out, RG_ERR_ARG, "rg_build_conservative_2d: out is NULL");
    *out = nullptr;
    rg_weights_s* W = new (std::nothrow) rg_weights_s();
    RG_CHECK(W, RG_ERR_ALLOC, "host allocation failed");
    cudaGetDevice(&W->device);
    int st = build_conservative_2d(d_xi, d_yi, nxi, nyi, d_xo, d_yo, nxo, nyo, d_w_in,
                                   (cudaStream_t)stream, W);
    if (st) {
        free_weights(W, (cudaStream_t)stream);
        return st;
    }
    *out = W;
    return RG_OK;
}

int rg_build_conservative_2d_batch(int64_t n, const double* const* d_xi, const double* const* d_yi,
                                   const int64_t* nxi, const int64_t* nyi, const double* const* d_xo,
                                   const double* const* d_yo, const int64_t* nxo, const int64_t* nyo,
                                   const double* const* d_w_in, rg_stream_t stream, rg_weights* out,
                                   int* status) {
    rg::NvtxRange nvtx_range("rg_build_conservative_2d_batch");
    RG_CHECK(n >= 1 && n < (1 << 24), RG_ERR_ARG, "rg_build_conservative_2d_batch: bad pair count %lld",
             (long long)n);
    RG_CHECK(d_xi && d_yi && nxi && nyi && d_xo && d_yo && nxo && nyo && out && status, RG_ERR_ARG,
             "rg_build_conservative_2d_batch: NULL argument");
    std::vector<PairSpec> pairs((size_t)n);
    std::vector<rg_weights_s*> W((size_t)n, nullptr);
    for (int64_t g = 0; g < n; g++) {
        out[g] = nullptr;
        status[g] = RG_ERR_ARG;
        pairs[g] = PairSpec{d_xi[g], d_yi[g], nxi[g], nyi[g], d_xo[g], d_yo[g], nxo[g], nyo[g],
                            d_w_in ? d_w_in[g] : nullptr};
    }
    int dev = 0;
    cudaGetDevice(&dev);
    for (int64_t g = 0; g < n; g++) {
        W[g] = new (std::nothrow) rg_weights_s();
        if (!W[g]) {
            for (int64_t k = 0; k < g; k++) delete W[k];
            RG_CHECK(false, RG_ERR_ALLOC, "host allocation failed");
        }
        W[g]->device = dev;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int st = build_batch(pairs.data(), (int)n, s, W.data(), status);
    for (int64_t g = 0; g < n; g++) {
        if (st == RG_OK && status[g] == RG_OK) {
            out[g] = W[g];
        } else {
            if (st != RG_OK) status[g] = st;
            free_weights(W[g], s);
        }
    }
    return st;
}

int rg_weights_from_coo(const int64_t* d_in, const int64_t* d_out, const double* d_val, int64_t nnz,
                        int64_t n_in, int64_t n_out, rg_stream_t stream, rg_weights* out) {
    rg::NvtxRange nvtx_range("rg_weights_from_coo");
    RG_CHECK(out, RG_ERR_ARG, "rg_weights_from_coo: out is NULL");
    RG_CHECK(nnz >= 0 && n_in >= 0 && n_out >= 0, RG_ERR_ARG, "rg_weights_from_coo: negative size");
    RG_CHECK(n_in < INT32_MAX && n_out < INT32_MAX, RG_ERR_UNSUPPORTED,
             "rg_weights_from_coo: more than 2^31 cells");
    *out = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    rg_weights_s* W = new (std::nothrow) rg_weights_s();
    RG_CHECK(W, RG_ERR_ALLOC, "host allocation failed");
    cudaGetDevice(&W->device);
    W->n_in = n_in;
    W->n_out = n_out;
    W->nnz = nnz;
    int32_t *in32 = nullptr, *out32 = nullptr;
    int64_t* pos = nullptr;
    uint32_t* perm = nullptr;
    unsigned* bad = nullptr;
    int st = RG_OK;
    do {
        if ((st = dalloc(&in32, (size_t)nnz, s))) break;
        if ((st = dalloc(&out32, (size_t)nnz, s))) break;
        if ((st = dalloc(&pos, (size_t)nnz, s))) break;
        if ((st = dalloc(&perm, (size_t)nnz, s))) break;
        if ((st = dalloc(&bad, 1, s))) break;
        if ((st = dalloc(&W->row_ptr, (size_t)n_out + 1, s))) break;
        if ((st = dalloc(&W->col, (size_t)nnz, s))) break;
        if ((st = dalloc(&W->val, (size_t)nnz, s))) break;
        cudaMemsetAsync(bad, 0, sizeof(unsigned), s);
        if (nnz > 0)
            normalise_coo<<<capped(nnz, 256), 256, 0, s>>>(d_in, d_out, nnz, n_in, n_out, in32, out32, pos,
                                                          bad);
        if (n_out > 0) {
            if ((st = bucket_sort(out32, pos, nnz, n_out, W->row_ptr, perm, nullptr, s))) break;
        } else {
            cudaMemsetAsync(W->row_ptr, 0, sizeof(int64_t), s);
        }
        if (nnz > 0) gather_csr<<<capped(nnz, 256), 256, 0, s>>>(perm, in32, d_val, nnz, W->col, W->val);
        unsigned hbad = 0;
        small_to_host(&hbad, bad, sizeof(unsigned), s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("rg_weights_from_coo: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }
        if (hbad) {
            set_error("rg_weights_from_coo: an index is out of range for the given shapes");
            st = RG_ERR_ARG;
        }
    } while (0);
    dfree(in32, s);
    dfree(out32, s);
    dfree(pos, s);
    dfree(perm, s);
    dfree(bad, s);
    if (st) {
        free_weights(W, s);
        return st;
    }
    *out = W;
    return RG_OK;
}

int rg_weights_info(rg_weights w, int64_t* nnz, int64_t* n_in, int64_t* n_out) {
    RG_CHECK(w, RG_ERR_ARG, "rg_weights_info: NULL handle");
    if (nnz) *nnz = w->nnz;
    if (n_in) *n_in = w->n_in;
    if (n_out) *n_out = w->n_out;
    return RG_OK;
}

int rg_weights_set_output_shape(rg_weights w, int64_t n0, int64_t n1) {
    RG_CHECK(w, RG_ERR_ARG, "rg_weights_set_output_shape: NULL handle");
    RG_CHECK(n0 * n1 == w->n_out, RG_ERR_ARG, "rg_weights_set_output_shape: %lld x %lld != %lld",
             (long long)n0, (long long)n1, (long long)w->n_out);
    std::lock_guard<std::mutex> lock(w->mu);
    if (w->out_shape0 == n0 && w->out_shape1 == n1) return RG_OK;
    RG_CHECK(!w->tiled_ready[0] && !w->tiled_ready[1], RG_ERR_ARG,
             "rg_weights_set_output_shape: the output tiling is fixed once a fast float32 apply has run");
    w->out_shape0 = n0;
    w->out_shape1 = n1;
    return RG_OK;
}

int rg_weights_export_coo(rg_weights w, int64_t* d_in, int64_t* d_out, double* d_val,
                          rg_stream_t stream) {
    rg::NvtxRange nvtx_range("rg_weights_export_coo");
    RG_CHECK(w, RG_ERR_ARG, "rg_weights_export_coo: NULL handle");
    if (w->nnz == 0) return RG_OK;
    cudaStream_t s = (cudaStream_t)stream;
    int32_t* row_of = nullptr;
    uint32_t* perm = nullptr;
    int64_t* col_ptr = nullptr;
    RG_TRY(column_order(w, &row_of, &perm, &col_ptr, s));
    gather_export<<<capped(w->nnz, 256), 256, 0, s>>>(perm, w->col, row_of, w->val, w->nnz, d_in, d_out,
                                                     d_val);
    dfree(row_of, s);
    dfree(perm, s);
    dfree(col_ptr, s);
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

int rg_weights_set_input_shape(rg_weights w, int64_t n0, int64_t n1) {
    RG_CHECK(w, RG_ERR_ARG, "rg_weights_set_input_shape: NULL handle");
    RG_CHECK(n0 * n1 == w->n_in, RG_ERR_ARG, "rg_weights_set_input_shape: %lld x %lld != %lld", (long long)n0,
             (long long)n1, (long long)w->n_in);
    std::lock_guard<std::mutex> lock(w->mu);
    if (w->in_shape0 == n0 && w->in_shape1 == n1) return RG_OK;
    RG_CHECK(w->box_state == 0, RG_ERR_ARG,
             "rg_weights_set_input_shape: the input tiling is fixed once a fast float32 apply has run");
    w->in_shape0 = n0;
    w->in_shape1 = n1;
    return RG_OK;
}

int rg_weights_check(rg_weights w, rg_stream_t stream) {
    RG_CHECK(w, RG_ERR_ARG, "rg_weights_check: NULL handle");
    RG_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    unsigned fl = 0;
    {
        std::lock_guard<std::mutex> lock(w->mu);
        if (!w->dflags) return RG_OK;
        RG_CUDA(cudaMemcpy(&fl, w->dflags, sizeof(unsigned), cudaMemcpyDeviceToHost));
    }
    RG_CHECK(!(fl & FLAG_TIMEOUT), RG_ERR_CUDA,
             "an earlier apply with this handle gave up waiting for its staged copies (its results are invalid)");
    return RG_OK;
}

int rg_weights_free(rg_weights w, rg_stream_t stream) {
    if (w) free_weights(w, (cudaStream_t)stream);
    return RG_OK;
}

int rg_apply(rg_weights w, const void* d_vin, int dtype_in, void* d_vout, int dtype_out, int64_t stack,
             int acc, rg_stream_t stream) {
    rg::NvtxRange nvtx_range("rg_apply");
    RG_CHECK(w, RG_ERR_ARG, "rg_apply: NULL handle");
    return apply_weights(w, false, d_vin, dtype_in, d_vout, dtype_out, stack, acc, (cudaStream_t)stream);
}

int rg_apply_host(rg_weights w, const void* h_vin, int dtype_in, void* h_vout, int dtype_out, int64_t stack,
                  int acc, int64_t chunk, rg_stream_t stream) {
    rg::NvtxRange nvtx_range("rg_apply_host");
    RG_CHECK(w, RG_ERR_ARG, "rg_apply_host: NULL handle");
    return apply_host(w, h_vin, dtype_in, h_vout, dtype_out, stack, acc, chunk, (cudaStream_t)stream);
}

int rg_apply_transpose(rg_weights w, const void* d_vout, int dtype_out, void* d_vin, int dtype_in,
                       int64_t stack, int acc, rg_stream_t stream) {
    rg::NvtxRange nvtx_range("rg_apply_transpose");
    RG_CHECK(w, RG_ERR_ARG, "rg_apply_transpose: NULL handle");
    return apply_weights(w, true, d_vout, dtype_out, d_vin, dtype_in, stack, acc, (cudaStream_t)stream);
}

int rg_cell_area_2d(const double* d_x, const double* d_y, int64_t nx, int64_t ny, double* d_area,
                    rg_stream_t stream) {
    RG_CHECK(nx >= 2 && ny >= 2, RG_ERR_ARG, "rg_cell_area_2d: need at least 2x2 vertices");
    return cell_area_2d(d_x, d_y, nx, ny, d_area, (cudaStream_t)stream);
}

int rg_cell_length_1d(const double* d_x, int64_t nd, int64_t n, double* d_len, rg_stream_t stream) {
    RG_CHECK(n >= 1, RG_ERR_ARG, "rg_cell_length_1d: empty grid");
    return cell_length_1d(d_x, nd, n, d_len, (cudaStream_t)stream);
}

int rg_locate_2d(const double* d_x, const double* d_y, int64_t nx, int64_t ny, const double* d_px,
                 const double* d_py, int64_t npts, int method, int64_t* d_i, int64_t* d_j,
                 rg_stream_t stream) {
    rg::NvtxRange nvtx_range("rg_locate_2d");
    RG_CHECK(nx >= 2 && ny >= 2, RG_ERR_ARG, "rg_locate_2d: need at least 2x2 vertices");
    RG_CHECK(method >= 0 && method <= 2, RG_ERR_ARG, "rg_locate_2d: unknown method %d", method);
    if (method == 2)
        return locate_2d_walk(d_x, d_y, nx, ny, d_px, d_py, npts, d_i, d_j, (cudaStream_t)stream);
    return locate_2d_exact(d_x, d_y, nx, ny, d_px, d_py, npts, method, d_i, d_j, (cudaStream_t)stream);
}

int rg_find_indices_1d(const double* d_xin, int64_t in_stride, int64_t m, const double* d_xout,
                       int64_t out_stride, int64_t n, int64_t nd, int method, int64_t fill_value,
                       int64_t* d_result, rg_stream_t stream) {
    rg::NvtxRange nvtx_range("rg_find_indices_1d");
    return find_indices_1d(d_xin, in_stride, m, d_xout, out_stride, n, nd, method, fill_value, d_result,
                           (cudaStream_t)stream);
}

int rg_multilinear_1d(const double* d_xin, int64_t in_stride, int64_t m, const double* d_xout,
                      const double* d_xout_search, int64_t out_stride, int64_t n, int64_t nd,
                      const double* d_w_in, int64_t w_stride, int bounds, int64_t* d_ind_in,
                      int64_t* d_ind_out, double* d_val, int64_t* h_n_outside, rg_stream_t stream) {
    rg::NvtxRange nvtx_range("rg_multilinear_1d");
    return multilinear_1d(d_xin, in_stride, m, d_xout, d_xout_search, out_stride, n, nd, d_w_in, w_stride,
                          bounds, d_ind_in, d_ind_out, d_val, h_n_outside, (cudaStream_t)stream);
}

int rg_conservative_1d(const double* d_xin, int64_t in_stride, int64_t m, const double* d_xout,
                       int64_t out_stride, int64_t n, int64_t nd, const double* d_w_in, int64_t w_stride,
                       int64_t cap, int64_t* d_ind_in, int64_t* d_ind_out, double* d_val, int64_t* d_count,
                       rg_stream_t stream) {
    rg::NvtxRange nvtx_range("rg_conservative_1d");
    return conservative_1d(d_xin, in_stride, m, d_xout, out_stride, n, nd, d_w_in, w_stride, cap, d_ind_in,
                           d_ind_out, d_val, d_count, (cudaStream_t)stream);
}

int rg_transpose_conservative_scale(const int64_t* d_in, const int64_t* d_out, const double* d_val,
                                    int64_t nnz, const double* d_vol_in, int64_t n_in,
                                    const double* d_vol_out, int64_t n_out, const double* d_w_in,
                                    double* d_result, rg_stream_t stream) {
    rg::NvtxRange nvtx_range("rg_transpose_conservative_scale");
    return transpose_conservative_scale(d_in, d_out, d_val, nnz, d_vol_in, n_in, d_vol_out, n_out, d_w_in,
                                        d_result, (cudaStream_t)stream);
}

}  // extern "C"

int rg_weights_device_bytes(rg_weights w, int64_t* bytes) {
    RG_CHECK(w && bytes, RG_ERR_ARG, "rg_weights_device_bytes: NULL argument");
    std::lock_guard<std::mutex> lock(w->mu);
    const int64_t nnz = w->nnz;
    int64_t b = (w->n_out + 1) * 8 + nnz * (4 + 8);
    if (w->val32) b += nnz * 4;
    if (w->t_row_ptr) b += (w->n_in + 1) * 8 + nnz * (4 + 8);
    if (w->t_val32) b += nnz * 4;
    for (int g = 0; g < 2; g++)
        if (w->tiled_ready[g]) b += (w->t_tiles + 1) * 8 + nnz * 2;  // list pointers + slots (lists are small)
    if (w->box_state == 1) b += w->box_patches * 8 + nnz * 6;  // origins; slot and float32 weight per entry
    if (w->ff_slot) b += nnz * 10;                              // compensated: slot, hi and lo per entry
    if (w->box_perm) b += w->box_patches * 256;
    if (w->ff_perm) b += w->box_patches * 256;
    *bytes = b;
    return RG_OK;
}

// Four independent 64-bit lanes over 8-byte words (multiply, rotate,
// multiply), folded together with the splitmix64 finaliser (Vigna).  Inputs
// above 4 MiB are cut into 1 MiB segments hashed on up to 8 host threads and
// combined in order, so the value does not depend on the thread count.
// Written for speed, not for resistance to chosen inputs.
namespace {
inline uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }
inline uint64_t fin64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
uint64_t hash_range(const unsigned char* p, int64_t n, uint64_t seed) {
    const uint64_t K1 = 0x9e3779b97f4a7c15ULL, K2 = 0xd6e8feb86659fd93ULL;
    uint64_t a[4] = {seed ^ K1, seed + K2, rotl64(seed, 17) ^ K2, ~seed};
    const int64_t total = n;
    while (n >= 32) {
        uint64_t w[4];
        memcpy(w, p, 32);
        for (int k = 0; k < 4; k++) a[k] = rotl64((a[k] ^ w[k]) * K1, 31) * K2;
        p += 32;
        n -= 32;
    }
    uint64_t tail[4] = {0, 0, 0, 0};
    memcpy(tail, p, (size_t)n);
    for (int k = 0; k < 4; k++) a[k] = rotl64((a[k] ^ tail[k]) * K1, 31) * K2;
    uint64_t h = fin64((uint64_t)total ^ seed);
    for (int k = 0; k < 4; k++) h = fin64(h ^ a[k]);
    return h;
}
// two hash_range values (seeds s0, s1) in one pass over the bytes
void hash_range2(const unsigned char* p, int64_t n, uint64_t s0, uint64_t s1, uint64_t* out) {
    const uint64_t K1 = 0x9e3779b97f4a7c15ULL, K2 = 0xd6e8feb86659fd93ULL;
    uint64_t a[4] = {s0 ^ K1, s0 + K2, rotl64(s0, 17) ^ K2, ~s0};
    uint64_t b[4] = {s1 ^ K1, s1 + K2, rotl64(s1, 17) ^ K2, ~s1};
    const int64_t total = n;
    while (n >= 32) {
        uint64_t w[4];
        memcpy(w, p, 32);
        for (int k = 0; k < 4; k++) {
            a[k] = rotl64((a[k] ^ w[k]) * K1, 31) * K2;
            b[k] = rotl64((b[k] ^ w[k]) * K1, 31) * K2;
        }
        p += 32;
        n -= 32;
    }
    uint64_t tail[4] = {0, 0, 0, 0};
    memcpy(tail, p, (size_t)n);
    for (int k = 0; k < 4; k++) {
        a[k] = rotl64((a[k] ^ tail[k]) * K1, 31) * K2;
        b[k] = rotl64((b[k] ^ tail[k]) * K1, 31) * K2;
    }
    uint64_t h0 = fin64((uint64_t)total ^ s0), h1 = fin64((uint64_t)total ^ s1);
    for (int k = 0; k < 4; k++) {
        h0 = fin64(h0 ^ a[k]);
        h1 = fin64(h1 ^ b[k]);
    }
    out[0] = h0;
    out[1] = h1;
}
}  // namespace

int rg_hash64x2(const void* h_data, int64_t nbytes, uint64_t seed0, uint64_t seed1, uint64_t* h_out) {
    RG_CHECK(h_out && nbytes >= 0 && (h_data || nbytes == 0), RG_ERR_ARG, "rg_hash64x2: bad argument");
    const unsigned char* p = (const unsigned char*)h_data;
    const int64_t SEG = 1 << 20;
    if (nbytes <= 4 * SEG) {
        hash_range2(p, nbytes, seed0, seed1, h_out);
        return RG_OK;
    }
    const int64_t nseg = (nbytes + SEG - 1) / SEG;
    std::vector<uint64_t> part0((size_t)nseg), part1((size_t)nseg);
    const int nthr = (int)(nseg < 16 ? nseg : 16);
    std::vector<std::thread> pool;
    for (int t = 0; t < nthr; t++)
        pool.emplace_back([&, t]() {
            for (int64_t k = t; k < nseg; k += nthr) {
                const int64_t len = nbytes - k * SEG < SEG ? nbytes - k * SEG : SEG;
                uint64_t h2[2];
                hash_range2(p + k * SEG, len, seed0 ^ (uint64_t)k, seed1 ^ (uint64_t)k, h2);
                part0[(size_t)k] = h2[0];
                part1[(size_t)k] = h2[1];
            }
        });
    for (auto& th : pool) th.join();
    h_out[0] = hash_range((const unsigned char*)part0.data(), nseg * 8, seed0 ^ (uint64_t)nbytes);
    h_out[1] = hash_range((const unsigned char*)part1.data(), nseg * 8, seed1 ^ (uint64_t)nbytes);
    return RG_OK;
}

int rg_hash64(const void* h_data, int64_t nbytes, uint64_t seed, uint64_t* h_out) {
    RG_CHECK(h_out && nbytes >= 0 && (h_data || nbytes == 0), RG_ERR_ARG, "rg_hash64: bad argument");
    const unsigned char* p = (const unsigned char*)h_data;
    const int64_t SEG = 1 << 20;
    if (nbytes <= 4 * SEG) {
        *h_out = hash_range(p, nbytes, seed);
        return RG_OK;
    }
    const int64_t nseg = (nbytes + SEG - 1) / SEG;
    std::vector<uint64_t> part((size_t)nseg);
    const int nthr = (int)(nseg < 8 ? nseg : 8);
    std::vector<std::thread> pool;
    for (int t = 0; t < nthr; t++)
        pool.emplace_back([&, t]() {
            for (int64_t k = t; k < nseg; k += nthr) {
                const int64_t len = nbytes - k * SEG < SEG ? nbytes - k * SEG : SEG;
                part[(size_t)k] = hash_range(p + k * SEG, len, seed ^ (uint64_t)k);
            }
        });
    for (auto& th : pool) th.join();
    *h_out = hash_range((const unsigned char*)part.data(), nseg * 8, seed ^ (uint64_t)nbytes);
    return RG_OK;
}
