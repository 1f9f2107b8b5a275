// Apply of device-resident weights to a stack of arrays:
//   values_output[d, o] = sum_k w[o, k] * values_input[d, col[o, k]]
// (regridding/_regrid/_regrid_from_weights.py:165-182).
//
// The matrix is stored by output row, so every output element is produced by
// exactly one thread with no atomics.  A block covers a 2D tile of output
// cells (8 x 32 when the output grid shape is known, so the input footprint of
// the block is compact and its gathers reuse L1/L2 lines) and a chunk of the
// stack; each thread keeps its row's first entries in registers and walks the
// stack chunk, so the weights are read once per chunk instead of once per
// array.
#include "common.cuh"

namespace rg {
namespace {

constexpr int APPLY_BLOCK = 256;
constexpr int CACHED = 8;  // row entries held in registers

template <typename T>
__device__ __forceinline__ T ldg_cast(const T* p) { return __ldg(p); }

struct Tile {
    int64_t n0, n1;  // output shape used for tiling (n0 = 1 for 1D tiling)
    int64_t tiles1;  // tiles along axis 1
    int t0, t1;      // tile extent
};

__device__ __forceinline__ int64_t tile_row(const Tile& T, int64_t tile, int tid) {
    int64_t ti = tile / T.tiles1, tj = tile % T.tiles1;
    int64_t i = ti * T.t0 + tid / T.t1;
    int64_t j = tj * T.t1 + tid % T.t1;
    if (i >= T.n0 || j >= T.n1) return -1;
    return i * T.n1 + j;
}

// MODE 0: exact double (mul then add, stored order), float64 output
// MODE 1: exact double update rounded to float32 after every entry (numpy's
//         in-place float32 output)
// MODE 2: fast, accumulate in the output type with FMA
template <typename Tin, typename Tout, int MODE, typename Tw>
__global__ void __launch_bounds__(APPLY_BLOCK)
    apply_kernel(const int64_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                 const Tw* __restrict__ val, Tile T, const Tin* __restrict__ vin, int64_t n_in,
                 Tout* __restrict__ vout, int64_t n_out, int64_t stack, int64_t chunk) {
    int64_t o = tile_row(T, blockIdx.x, threadIdx.x);
    if (o < 0) return;
    int64_t d0 = (int64_t)blockIdx.y * chunk;
    int64_t d1 = d0 + chunk < stack ? d0 + chunk : stack;
    int64_t s = row_ptr[o], e = row_ptr[o + 1];
    int nk = (int)(e - s);
    int32_t c[CACHED];
    Tw w[CACHED];
#pragma unroll
    for (int k = 0; k < CACHED; k++) {
        c[k] = k < nk ? col[s + k] : 0;
        w[k] = k < nk ? val[s + k] : (Tw)0;
    }
    for (int64_t d = d0; d < d1; d++) {
        const Tin* a = vin + d * n_in;
        if (MODE == 0) {
            double acc = 0.0;
#pragma unroll
            for (int k = 0; k < CACHED; k++)
                if (k < nk) acc = __dadd_rn(acc, __dmul_rn((double)w[k], (double)ldg_cast(a + c[k])));
            for (int64_t k = s + CACHED; k < e; k++)
                acc = __dadd_rn(acc, __dmul_rn((double)val[k], (double)ldg_cast(a + col[k])));
            vout[d * n_out + o] = (Tout)acc;
        } else if (MODE == 1) {
            float acc = 0.0f;
#pragma unroll
            for (int k = 0; k < CACHED; k++)
                if (k < nk)
                    acc = (float)__dadd_rn((double)acc, __dmul_rn((double)w[k], (double)ldg_cast(a + c[k])));
            for (int64_t k = s + CACHED; k < e; k++)
                acc = (float)__dadd_rn((double)acc, __dmul_rn((double)val[k], (double)ldg_cast(a + col[k])));
            vout[d * n_out + o] = (Tout)acc;
        } else {
            Tout acc = (Tout)0;
#pragma unroll
            for (int k = 0; k < CACHED; k++)
                if (k < nk) acc = fma((Tout)w[k], (Tout)ldg_cast(a + c[k]), acc);
            for (int64_t k = s + CACHED; k < e; k++) acc = fma((Tout)val[k], (Tout)ldg_cast(a + col[k]), acc);
            vout[d * n_out + o] = acc;
        }
    }
}

__global__ void to_f32(const double* a, float* b, int64_t n) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        b[k] = (float)a[k];
}

template <typename Tin, typename Tout, int MODE, typename Tw>
int launch(const int64_t* row_ptr, const int32_t* col, const Tw* val, int64_t n_rows,
           int64_t shape0, int64_t shape1, const void* vin, int64_t n_in, void* vout, int64_t stack,
           cudaStream_t s) {
    Tile T;
    if (shape0 > 0 && shape1 > 0 && shape0 * shape1 == n_rows && shape1 >= 32) {
        T.n0 = shape0;
        T.n1 = shape1;
        T.t0 = 8;
        T.t1 = 32;
    } else {
        T.n0 = 1;
        T.n1 = n_rows;
        T.t0 = 1;
        T.t1 = APPLY_BLOCK;
    }
    T.tiles1 = (T.n1 + T.t1 - 1) / T.t1;
    int64_t tiles = ((T.n0 + T.t0 - 1) / T.t0) * T.tiles1;
    // stack chunk: enough blocks to fill the GPU, at most 65535 along y
    int64_t chunk = 16;
    if (tiles >= 4 * 152 * 8) chunk = 64;
    if ((stack + chunk - 1) / chunk > 65535) chunk = (stack + 65534) / 65535;
    int64_t chunks = (stack + chunk - 1) / chunk;
    RG_CHECK(tiles < 0x7fffffff, RG_ERR_UNSUPPORTED, "apply: too many output cells");
    dim3 grid((unsigned)tiles, (unsigned)chunks);
    apply_kernel<Tin, Tout, MODE, Tw><<<grid, APPLY_BLOCK, 0, s>>>(
        row_ptr, col, val, T, (const Tin*)vin, n_in, (Tout*)vout, n_rows, stack, chunk);
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

int apply_csr(const int64_t* row_ptr, const int32_t* col, const double* val, const float* val32,
              int64_t nnz, int64_t n_rows, int64_t n_cols, int64_t shape0, int64_t shape1,
              const void* vin, int dtype_in, void* vout, int dtype_out, int64_t stack, int acc,
              cudaStream_t s) {
    RG_CHECK(dtype_in == RG_F32 || dtype_in == RG_F64, RG_ERR_ARG, "apply: bad input dtype");
    RG_CHECK(dtype_out == RG_F32 || dtype_out == RG_F64, RG_ERR_ARG, "apply: bad output dtype");
    RG_CHECK(acc == RG_ACC_EXACT || acc == RG_ACC_FAST || acc == RG_ACC_COMPENSATED, RG_ERR_ARG,
             "apply: bad accumulation mode");
    if (stack <= 0 || n_rows <= 0) return RG_OK;
    if (acc != RG_ACC_FAST) {  // exact, or compensated where the staged kernel does not take the call
        if (dtype_out == RG_F64) {
            if (dtype_in == RG_F32)
                return launch<float, double, 0, double>(row_ptr, col, val, n_rows, shape0, shape1, vin, n_cols,
                                                        vout, stack, s);
            return launch<double, double, 0, double>(row_ptr, col, val, n_rows, shape0, shape1, vin, n_cols,
                                                     vout, stack, s);
        }
        if (dtype_in == RG_F32)
            return launch<float, float, 1, double>(row_ptr, col, val, n_rows, shape0, shape1, vin, n_cols, vout,
                                                   stack, s);
        return launch<double, float, 1, double>(row_ptr, col, val, n_rows, shape0, shape1, vin, n_cols, vout,
                                                stack, s);
    }
    if (dtype_out == RG_F64) {
        if (dtype_in == RG_F32)
            return launch<float, double, 2, double>(row_ptr, col, val, n_rows, shape0, shape1, vin, n_cols, vout,
                                                    stack, s);
        return launch<double, double, 2, double>(row_ptr, col, val, n_rows, shape0, shape1, vin, n_cols, vout,
                                                 stack, s);
    }
    // float32 output, fast: the weights rounded to float once (made by the caller)
    if (dtype_in == RG_F32)
        return launch<float, float, 2, float>(row_ptr, col, val32, n_rows, shape0, shape1, vin, n_cols, vout,
                                              stack, s);
    return launch<double, float, 2, float>(row_ptr, col, val32, n_rows, shape0, shape1, vin, n_cols, vout,
                                           stack, s);
}

}  // namespace

int tiled_lists_for(rg_weights_s* W, const float* vin, cudaStream_t s, int* g, bool* made);
int apply_tiled(const rg_weights_s* W, int g, const float* vin, float* vout, int64_t stack, cudaStream_t s);
bool box_usable(const rg_weights_s* W, const float* vin, int64_t stack);
int box_lists_for(rg_weights_s* W, cudaStream_t s, bool* made);
int box_perm_for(rg_weights_s* W, cudaStream_t s, bool* made);
int ff_lists_for(rg_weights_s* W, cudaStream_t s, bool* made);
int apply_box(const rg_weights_s* W, const float* vin, float* vout, int64_t stack, cudaStream_t s);
int apply_box_exact(const rg_weights_s* W, const float* vin, double* vout, int64_t stack, cudaStream_t s);
int apply_box_ff(const rg_weights_s* W, const float* vin, double* vout, int64_t stack, cudaStream_t s);
int tune_box_fast(rg_weights_s* W, const float* vin, float* vout, int64_t stack, cudaStream_t s);
int tune_box_ff(rg_weights_s* W, const float* vin, double* vout, int64_t stack, cudaStream_t s);
int rows_usable(rg_weights_s* W, const float* vin, int64_t stack, cudaStream_t s, bool* made, bool* ok);
int apply_rows_launch(const rg_weights_s* W, const float* vin, float* vout, int64_t stack, cudaStream_t s);
int ensure_transposed(rg_weights_s* W, cudaStream_t s);

// Every apply goes through here.  The per-handle state an apply needs beyond
// the CSR (the transposed CSR, the float32 copy of the weights, the warp-tile
// lists) is made on first use under the handle's mutex and finished (the
// stream synchronised) before the lock is released, so calls from other
// threads and streams only ever see complete state.
int apply_weights(rg_weights_s* W, bool transposed, const void* vin, int dtype_in, void* vout,
                  int dtype_out, int64_t stack, int acc, cudaStream_t s) {
    RG_CHECK(dtype_in == RG_F32 || dtype_in == RG_F64, RG_ERR_ARG, "apply: bad input dtype");
    RG_CHECK(dtype_out == RG_F32 || dtype_out == RG_F64, RG_ERR_ARG, "apply: bad output dtype");
    RG_CHECK(acc == RG_ACC_EXACT || acc == RG_ACC_FAST || acc == RG_ACC_COMPENSATED, RG_ERR_ARG,
             "apply: bad accumulation mode");
    if (stack <= 0) return RG_OK;
    // the bandwidth path: float32 in and out, input staged in shared memory (by
    // tensor-map copies when the input grid shape allows, else by the warps)
    const bool tiled = !transposed && acc == RG_ACC_FAST && dtype_in == RG_F32 && dtype_out == RG_F32 &&
                       W->n_out > 0 && W->nnz > 0;
    // the exact float64 apply of a float32 stack stages input boxes too
    const bool exact_box = !transposed && acc == RG_ACC_EXACT && dtype_in == RG_F32 && dtype_out == RG_F64 &&
                           W->n_out > 0 && W->nnz > 0;
    // the compensated apply: float32 stack, float64 output, float-float sums
    const bool ff_box = !transposed && acc == RG_ACC_COMPENSATED && dtype_in == RG_F32 && dtype_out == RG_F64 &&
                        W->n_out > 0 && W->nnz > 0;
    // (the patch lists keep a float32 copy of the weights in gather order)
    const bool need32 = ((acc == RG_ACC_FAST && dtype_out == RG_F32) || exact_box || ff_box) && W->nnz > 0;
    int g = 0;
    bool use_box = false, use_rows = false, use_box_exact = false, use_box_ff = false;
    {
        std::lock_guard<std::mutex> lock(W->mu);
        bool made = false;
        if (transposed && W->t_row_ptr == nullptr) {
            RG_TRY(ensure_transposed(W, s));
            made = true;
        }
        float** v32 = transposed ? &W->t_val32 : &W->val32;
        if (need32 && *v32 == nullptr) {
            RG_TRY(dalloc(v32, (size_t)W->nnz, s));
            to_f32<<<grid_for(W->nnz, 256) > 8192 ? 8192 : grid_for(W->nnz, 256), 256, 0, s>>>(
                transposed ? W->t_val : W->val, *v32, W->nnz);
            made = true;
        }
        if (tiled && box_usable(W, (const float*)vin, stack)) {
            RG_TRY(box_lists_for(W, s, &made));
            use_box = W->box_state == 1;
            if (use_box && W->box_cfg[stack_class(stack)] == -1) {
                if (made) RG_CUDA(cudaStreamSynchronize(s));
                made = false;
                RG_TRY(tune_box_fast(W, (const float*)vin, (float*)vout, stack, s));
            }
            use_box = use_box && W->box_cfg[stack_class(stack)] >= 0;
        }
        if (exact_box && box_usable(W, (const float*)vin, stack)) {
            RG_TRY(box_lists_for(W, s, &made));
            use_box_exact = W->box_state == 1;
            if (use_box_exact) RG_TRY(box_perm_for(W, s, &made));
        }
        if (ff_box && box_usable(W, (const float*)vin, stack)) {
            RG_TRY(box_lists_for(W, s, &made));
            use_box_ff = W->box_state == 1;
            if (use_box_ff) RG_TRY(ff_lists_for(W, s, &made));
            if (use_box_ff && W->box_cfg_ff[stack_class(stack)] == -1) {
                if (made) RG_CUDA(cudaStreamSynchronize(s));
                made = false;
                RG_TRY(tune_box_ff(W, (const float*)vin, (double*)vout, stack, s));
            }
            use_box_ff = use_box_ff && W->box_cfg_ff[stack_class(stack)] >= 0;
        }
        if (tiled && !use_box) RG_TRY(rows_usable(W, (const float*)vin, stack, s, &made, &use_rows));
        if (tiled && !use_box && !use_rows) RG_TRY(tiled_lists_for(W, (const float*)vin, s, &g, &made));
        if (made) RG_CUDA(cudaStreamSynchronize(s));
    }
    if (use_rows) return apply_rows_launch(W, (const float*)vin, (float*)vout, stack, s);
    if (use_box_exact) {
        const int st = apply_box_exact(W, (const float*)vin, (double*)vout, stack, s);
        if (st != RG_ERR_UNSUPPORTED) return st;
    }
    if (use_box_ff) {
        const int st = apply_box_ff(W, (const float*)vin, (double*)vout, stack, s);
        if (st != RG_ERR_UNSUPPORTED) return st;
    }
    if (use_box) {
        const int st = apply_box(W, (const float*)vin, (float*)vout, stack, s);
        if (st != RG_ERR_UNSUPPORTED) return st;
        // the tuned configuration does not take this call (fewer slices than
        // a stage): the warp-staged kernel does, with its own lists
        std::lock_guard<std::mutex> lock(W->mu);
        bool made = false;
        RG_TRY(tiled_lists_for(W, (const float*)vin, s, &g, &made));
        if (made) RG_CUDA(cudaStreamSynchronize(s));
    }
    if (tiled) return apply_tiled(W, g, (const float*)vin, (float*)vout, stack, s);
    if (!transposed)
        return apply_csr(W->row_ptr, W->col, W->val, W->val32, W->nnz, W->n_out, W->n_in, W->out_shape0,
                         W->out_shape1, vin, dtype_in, vout, dtype_out, stack, acc, s);
    return apply_csr(W->t_row_ptr, W->t_col, W->t_val, W->t_val32, W->nnz, W->n_in, W->n_out, 0, 0, vin,
                     dtype_in, vout, dtype_out, stack, acc, s);
}

}  // namespace rg

// ---------------------------------------------------------------------------
// apply with the stack in host memory: the stack is cut into chunks that are
// copied in, applied and copied out on three streams, so the two copy
// directions and the kernels overlap (double-buffered staging in HBM).
// ---------------------------------------------------------------------------
namespace rg {

int apply_host(rg_weights_s* W, const void* h_vin, int dtype_in, void* h_vout, int dtype_out,
               int64_t stack, int acc, int64_t chunk, cudaStream_t s) {
    RG_CHECK(dtype_in == RG_F32 || dtype_in == RG_F64, RG_ERR_ARG, "apply_host: bad input dtype");
    RG_CHECK(dtype_out == RG_F32 || dtype_out == RG_F64, RG_ERR_ARG, "apply_host: bad output dtype");
    if (stack <= 0) return RG_OK;
    const size_t bin = (dtype_in == RG_F32 ? 4 : 8) * (size_t)W->n_in;
    const size_t bout = (dtype_out == RG_F32 ? 4 : 8) * (size_t)W->n_out;
    if (chunk <= 0) {
        // about 128 MB of input per chunk, at least one slice
        chunk = (int64_t)((128u << 20) / (bin ? bin : 1));
        if (chunk < 1) chunk = 1;
    }
    if (chunk > stack) chunk = stack;
    const int64_t nchunks = (stack + chunk - 1) / chunk;

    cudaStream_t sin = nullptr, sout = nullptr;
    cudaEvent_t ev[2 * 3] = {};
    char* dbuf[4] = {};
    int st = RG_OK;
    do {
        if (cudaStreamCreateWithFlags(&sin, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&sout, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            set_error("apply_host: stream creation failed");
            st = RG_ERR_CUDA;
            break;
        }
        for (int k = 0; k < 6; k++)
            if (cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming) != cudaSuccess) {
                cudaGetLastError();
                set_error("apply_host: event creation failed");
                st = RG_ERR_CUDA;
            }
        if (st) break;
        for (int b = 0; b < 2; b++) {
            if ((st = dalloc(&dbuf[b], bin * chunk, s))) break;
            if ((st = dalloc(&dbuf[2 + b], bout * chunk, s))) break;
        }
        if (st) break;
        // ev[0..1]: input buffer b consumed by the kernel; ev[2..3]: output
        // buffer b copied out; ev[4]: input copy of the current chunk landed;
        // ev[5]: kernel of the current chunk done
        cudaEventRecord(ev[0], s);
        cudaEventRecord(ev[1], s);
        cudaEventRecord(ev[2], s);
        cudaEventRecord(ev[3], s);
        for (int64_t c = 0; c < nchunks && st == RG_OK; c++) {
            int b = (int)(c & 1);
            int64_t d0 = c * chunk, nd = stack - d0 < chunk ? stack - d0 : chunk;
            cudaStreamWaitEvent(sin, ev[b], 0);
            cudaMemcpyAsync(dbuf[b], (const char*)h_vin + d0 * bin, bin * nd, cudaMemcpyHostToDevice, sin);
            cudaEventRecord(ev[4], sin);
            cudaStreamWaitEvent(s, ev[4], 0);
            cudaStreamWaitEvent(s, ev[2 + b], 0);
            st = apply_weights(W, false, dbuf[b], dtype_in, dbuf[2 + b], dtype_out, nd, acc, s);
            cudaEventRecord(ev[b], s);
            cudaEventRecord(ev[5], s);
            cudaStreamWaitEvent(sout, ev[5], 0);
            cudaMemcpyAsync((char*)h_vout + d0 * bout, dbuf[2 + b], bout * nd, cudaMemcpyDeviceToHost, sout);
            cudaEventRecord(ev[2 + b], sout);
        }
        // the caller's stream completes after the last copy out
        cudaStreamWaitEvent(s, ev[2], 0);
        cudaStreamWaitEvent(s, ev[3], 0);
        cudaError_t e = cudaGetLastError();
        if (st == RG_OK && e != cudaSuccess) {
            set_error("apply_host: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
        }
    } while (0);
    for (int b = 0; b < 4; b++) dfree(dbuf[b], s);
    for (int k = 0; k < 6; k++)
        if (ev[k]) cudaEventDestroy(ev[k]);
    if (sin) cudaStreamDestroy(sin);
    if (sout) cudaStreamDestroy(sout);
    return st;
}

}  // namespace rg
