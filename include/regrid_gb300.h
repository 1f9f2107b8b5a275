/*
 * regrid_gb300 — C ABI of the GB300 (sm_103a) regridding kernels.
 *
 * The upstream package (sun-data/regridding) is a Python + Numba library with
 * no C interface; each entry point below replaces one of its compiled loops,
 * cited beside it as upstream-path:line.  The Python package
 * `regridding_gb300` binds these symbols with ctypes and keeps the upstream
 * Python signatures on top.
 *
 * Conventions
 *  - Every pointer argument named d_* is a device pointer on the current
 *    device; h_* pointers are host memory.  Arrays are C-contiguous.
 *  - Every function returns an RG_* status (0 = success).  On failure a
 *    message is available from rg_last_error() in the calling thread.
 *  - Work is enqueued on the given stream.  Functions that must return a
 *    size to the host (the number of weights of a build) synchronise that
 *    stream; this is stated beside them.  All others are asynchronous.
 *  - Distinct handles may be used concurrently from different host threads
 *    on different streams.  A handle must not be freed while work that uses
 *    it is in flight.
 *  - There is no CPU fallback: without a usable GPU every call fails with
 *    RG_ERR_CUDA.
 */
#ifndef REGRID_GB300_H
#define REGRID_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* rg_stream_t; /* == cudaStream_t */

/* status codes */
#define RG_OK 0
#define RG_ERR_ARG 1        /* invalid argument (the upstream raises ValueError) */
#define RG_ERR_CUDA 2       /* CUDA runtime failure */
#define RG_ERR_ALLOC 3      /* device allocation failed */
#define RG_ERR_WALK 4       /* a sweep walk hit its step cap or was seated outside the grid */
#define RG_ERR_UNSUPPORTED 5

/* value dtypes */
#define RG_F32 0
#define RG_F64 1

/* apply accumulation modes */
#define RG_ACC_EXACT 0 /* double, multiply then add, entries in stored order: bit-identical to upstream */
#define RG_ACC_FAST 1  /* accumulate in the output dtype with fused multiply-add */
/* float32 input, float64 output: every product and partial sum carried as an
 * unevaluated pair of floats (error-free products by FMA, Knuth's two-sum) on
 * the FP32 pipe, the pair added in double at the end.  Result within
 * (1.1e-14 + (n + 2)^2 * 3.6e-15) * sum_k |w_k x_k| of the exact sum for rows
 * of n entries (checked to 1e-12 relative against the upstream float64 apply).
 * A float32 partial sum that overflows, or a non-finite input or weight,
 * sends that output and slice to the exact float64 sum instead.
 * Every other dtype combination computes as RG_ACC_EXACT. */
#define RG_ACC_COMPENSATED 2

/* multilinear bounds (upstream `bounds` argument) */
#define RG_BOUNDS_EXTRAPOLATE 0
#define RG_BOUNDS_NAN 1
#define RG_BOUNDS_RAISE 2

typedef struct rg_weights_s* rg_weights; /* device-resident sparse weights of one element */

/* Library version (major * 10000 + minor * 100 + patch). */
int rg_version(void);

/* Copies the calling thread's last error message into buf (always
 * NUL-terminated); returns the message length. */
int rg_last_error(char* buf, size_t n);

/* ---------------------------------------------------------------- weights */

/* Conservative (Ramshaw edge-sweep) weights between two logically
 * rectangular 2D vertex grids of one orthogonal element.
 * Replaces weights_conservative_2d,
 *   regridding/_weights/_weights_conservative_2d/_weights_conservative_2d.py:76-126,
 * together with the per-element coalescing of _coalesce,
 *   regridding/_weights/_weights_arrays.py:44-73.
 * Grids are (nx, ny) float64 arrays; d_w_in is NULL or (nxi-1, nyi-1).
 * The output grid must already carry the upstream seeded perturbation if one
 * is wanted (the host draws it).  Synchronises `stream` (twice: the raw and
 * the merged entry counts size the buffers).  On success *out owns a new
 * handle. */
int rg_build_conservative_2d(const double* d_xi, const double* d_yi, int64_t nxi, int64_t nyi,
                             const double* d_xo, const double* d_yo, int64_t nxo, int64_t nyo,
                             const double* d_w_in, rg_stream_t stream, rg_weights* out);

/* Sweep segments per chunk of the parallel walk in conservative builds
 * (process-wide; default 32; 0 walks whole lines in one thread each).  The
 * RG_SWEEP_CHUNK environment variable overrides it.  Results do not depend on
 * it, only the build time does (the chunked walk repairs every chunk whose
 * guessed start differs from its predecessor's end).  No upstream
 * counterpart. */
int rg_set_sweep_chunk(int64_t segments);

/* Conservative 2D weights of n independent grid pairs built together: every
 * stage runs once over all pairs (their sweep lines, chunks and output rows
 * concatenated into one work queue), so the batch synchronises with the host
 * a fixed number of times whatever n is.  Arrays of n device pointers / sizes
 * as in rg_build_conservative_2d (d_w_in may be NULL, or hold NULL entries).
 * out[g] receives pair g's handle and status[g] its status: a pair whose
 * sweep fails (degenerate grids) gets RG_ERR_WALK and a NULL handle without
 * affecting the others.  Returns RG_OK when the batch ran.  Results are bit
 * for bit those of rg_build_conservative_2d on each pair.  No upstream
 * counterpart (the upstream loops over elements in Python:
 * regridding/_weights/_weights_conservative.py:110-139). */
int rg_build_conservative_2d_batch(int64_t n, const double* const* d_xi, const double* const* d_yi,
                                   const int64_t* nxi, const int64_t* nyi, const double* const* d_xo,
                                   const double* const* d_yo, const int64_t* nxo, const int64_t* nyo,
                                   const double* const* d_w_in, rg_stream_t stream, rg_weights* out,
                                   int* status);

/* Weights from entries in the upstream saved layout (one element):
 * indices_input, indices_output (int64, negative values count from the end as
 * in numpy), values (float64).  Entries of one output are applied in the
 * order given, as regridding/_regrid/_regrid_from_weights.py:179-182 does.
 * Synchronises nothing. */
int rg_weights_from_coo(const int64_t* d_in, const int64_t* d_out, const double* d_val, int64_t nnz,
                        int64_t n_in, int64_t n_out, rg_stream_t stream, rg_weights* out);

/* Number of stored entries and the matrix shape. */
int rg_weights_info(rg_weights w, int64_t* nnz, int64_t* n_in, int64_t* n_out);

/* Record the 2D shape of the output cells (rows of the matrix) so the apply
 * can tile them in two dimensions.  Optional; the shape cannot change once a
 * fast float32 apply has run with the handle (RG_ERR_ARG).
 *
 * Handles may be shared between threads and streams: the state an apply
 * makes on first use (float32 weights, tile lists, transposed CSR) is made
 * under a per-handle lock and completed before other calls can see it.
 * Freeing a handle while another call uses it is the caller's error. */
int rg_weights_set_output_shape(rg_weights w, int64_t n0, int64_t n1);

/* Entries in the upstream saved layout: unique (input, output) pairs sorted by
 * (input, output), as returned by regridding/_weights/_weights.py:186.
 * Buffers hold nnz entries each. */
int rg_weights_export_coo(rg_weights w, int64_t* d_in, int64_t* d_out, double* d_val,
                          rg_stream_t stream);

/* Record the 2D shape of the input cells (columns of the matrix), which
 * lets the fast float32 apply stage input boxes with tensor-map copies.
 * Optional (weights built by rg_build_conservative_2d have it); fixed once a
 * fast float32 apply has run (RG_ERR_ARG). */
int rg_weights_set_input_shape(rg_weights w, int64_t n0, int64_t n1);

/* Synchronise `stream` and report a failure that an earlier asynchronous
 * apply with this handle recorded on the device: a staged copy that did not
 * complete within its bounded wait (RG_ERR_CUDA; the results of that apply
 * are invalid).  RG_OK when there was none. */
int rg_weights_check(rg_weights w, rg_stream_t stream);

/* Free a handle (stream ordered on `stream`). */
int rg_weights_free(rg_weights w, rg_stream_t stream);

/* --------------------------------------------------------------- apply */

/* values_output[d, o] = sum_k w[o,k] * values_input[d, col[o,k]] for d < stack.
 * Replaces _regrid_from_weights, regridding/_regrid/_regrid_from_weights.py:165-182.
 * d_vin is (stack, n_in) of dtype_in (RG_F32/RG_F64), d_vout is
 * (stack, n_out) of dtype_out.  acc = RG_ACC_EXACT reproduces the upstream
 * float64 result bit for bit (dtype_out must be RG_F64, or RG_F32 for the
 * upstream in-place float32 output, which rounds after every update);
 * RG_ACC_FAST accumulates in dtype_out with FMA; RG_ACC_COMPENSATED gives a
 * float64 result within 1e-12 of the upstream's for float32 input, about 5x
 * faster than RG_ACC_EXACT on GB300 (see its definition above).
 * The first fast or compensated apply of a handle (which builds its tile
 * lists and entry orders) and its first in each stack size class (1, 2-3,
 * 4-7, ..., 64 and more slices: the autotuner times its configurations on
 * that call, unless an earlier handle of the same kind was tuned) synchronise
 * `stream`; later applies are asynchronous. */
int rg_apply(rg_weights w, const void* d_vin, int dtype_in, void* d_vout, int dtype_out,
             int64_t stack, int acc, rg_stream_t stream);

/* rg_apply with the stack in HOST memory: h_vin (stack, n_in) and h_vout
 * (stack, n_out).  The stack is processed in chunks of `chunk` slices (0 =
 * automatic, about 128 MB of input per chunk) that are copied in, applied
 * and copied out on separate streams so copies in both directions overlap
 * the kernels.  This is the entry point for callers that hold their arrays
 * on the host, as the upstream regrid_from_weights
 * (regridding/_regrid/_regrid_from_weights.py:12-162) does.  Page-locked
 * host buffers give full link bandwidth.  Asynchronous: h_vout is complete
 * once `stream` has been synchronised. */
int rg_apply_host(rg_weights w, const void* h_vin, int dtype_in, void* h_vout, int dtype_out,
                  int64_t stack, int acc, int64_t chunk, rg_stream_t stream);

/* The same with the transposed matrix (rows = input cells):
 * values_input[d, i] = sum_o w[o, i] * values_output[d, o].  This is the
 * apply of transpose_weights(),
 * regridding/_weights/_weights_transposed/_weights_transposed.py:13-50, and
 * the backward of the apply with respect to the values.  The first call
 * builds the transposed index (stream ordered). */
int rg_apply_transpose(rg_weights w, const void* d_vout, int dtype_out, void* d_vin, int dtype_in,
                       int64_t stack, int acc, rg_stream_t stream);

/* ------------------------------------------------------------ geometry */

/* Cell areas of a 2D vertex grid: grid_volume,
 * regridding/_weights/_weights_conservative_2d/_grids.py:50-140 (bit-identical). */
int rg_cell_area_2d(const double* d_x, const double* d_y, int64_t nx, int64_t ny, double* d_area,
                    rg_stream_t stream);

/* Cell lengths of a batch of 1D grids: cell_length,
 * regridding/_weights/_weights_conservative_1d/_grids.py:10-35. d_x is (nd, n),
 * d_len is (nd, n-1). */
int rg_cell_length_1d(const double* d_x, int64_t nd, int64_t n, double* d_len, rg_stream_t stream);

/* Locate points in a curvilinear 2D grid: the lowest-index cell containing
 * each point, (INT64_MAX, INT64_MAX) outside.  method 0 = exhaustive order
 * (index_of_point_brute, _grids.py:218-279); method 1 = the secant iteration
 * with the local ascending search (index_of_point_secant, _grids.py:352-463);
 * method 2 = grid walk (a new fast path with the exhaustive-order result on
 * grids whose cells do not overlap). */
int rg_locate_2d(const double* d_x, const double* d_y, int64_t nx, int64_t ny, const double* d_px,
                 const double* d_py, int64_t npts, int method, int64_t* d_i, int64_t* d_j,
                 rg_stream_t stream);

/* Largest point count of one rg_locate_2d_noalloc call. */
#define RG_LOCATE_NOALLOC_MAX_POINTS 1048576

/* rg_locate_2d with method 2 (grid walk) that allocates no device memory.
 * This entry point has no counterpart in the upstream package.  It serves
 * callers that cannot allocate at call time: processes whose device memory is
 * owned by another allocator or a fixed budget, and latency-critical loops
 * that must not meet an allocation's implicit synchronisation or an
 * out-of-memory failure mid-stream.  The scratch it needs (the points the walk
 * hands to the exhaustive fallback) is a static device array of
 * 8 * (32 + RG_LOCATE_NOALLOC_MAX_POINTS) bytes (about 8 MiB) that every GPU
 * which loads the library holds until the process exits.  The first call on
 * each device looks up that array's device address (with the device
 * current); make that first call before capturing the stream into a graph.
 * At most RG_LOCATE_NOALLOC_MAX_POINTS points per call (RG_ERR_ARG beyond).
 * Every call on a device shares the one array, so calls that overlap on the
 * GPU (different streams, or host threads) race and must be serialised.
 * The looked-up address is kept until the process exits: resetting a device
 * (cudaDeviceReset) after the first call on it is not supported.
 * Points the walk cannot place (every point outside the grid) go to a
 * fallback that scans all 2 (nx + ny - 2) boundary edges with one warp per
 * point, about (nx + ny) / 16 edge tests per lane: with many points outside
 * a large grid this costs far more than rg_locate_2d, whose fallback bins
 * the boundary edges by y.
 * Results equal rg_locate_2d with method 2. */
int rg_locate_2d_noalloc(const double* d_x, const double* d_y, int64_t nx, int64_t ny,
                         const double* d_px, const double* d_py, int64_t npts, int64_t* d_i,
                         int64_t* d_j, rg_stream_t stream);

/* 1D find_indices on a batch of nd rows.  method 0 = brute
 * (_find_indices_brute_1d, regridding/_find_indices/_find_indices_brute.py:24-51),
 * method 1 = searchsorted (_find_indices_searchsorted_1d,
 * regridding/_find_indices/_find_indices_searchsorted.py:24-62).  Row d of the
 * inputs starts at d * x_stride (a stride of 0 broadcasts one row). */
int rg_find_indices_1d(const double* d_xin, int64_t in_stride, int64_t m, const double* d_xout,
                       int64_t out_stride, int64_t n, int64_t nd, int method, int64_t fill_value,
                       int64_t* d_result, rg_stream_t stream);

/* Multilinear weights of nd 1D rows: find_indices(searchsorted), the bounds
 * resolution of _weights_from_indices_multilinear
 * (regridding/_weights/_weights_multilinear.py:101-119) and
 * _weights_from_indices_multilinear_1d (:142-206), followed by the per-element
 * coalescing (_coalesce).  Outputs are (nd, 2n) arrays in the upstream saved
 * layout of each element.  With RG_BOUNDS_RAISE, *h_n_outside receives the
 * number of outside points (synchronises) and nothing else is valid if it is
 * nonzero.  d_w_in is NULL or rows of m values with stride w_stride.
 * d_xout_search is NULL or the output coordinates used for the cell search
 * (the upstream searches with the unperturbed coordinates and computes the
 * weights from the perturbed ones when `perturb` is set); it shares
 * out_stride with d_xout. */
int rg_multilinear_1d(const double* d_xin, int64_t in_stride, int64_t m, const double* d_xout,
                      const double* d_xout_search, int64_t out_stride, int64_t n, int64_t nd,
                      const double* d_w_in,
                      int64_t w_stride, int bounds, int64_t* d_ind_in, int64_t* d_ind_out,
                      double* d_val, int64_t* h_n_outside, rg_stream_t stream);

/* Conservative 1D weights of nd rows: _weights_conservative_1d,
 * regridding/_weights/_weights_conservative_1d/_weights_conservative_1d.py:59-318,
 * followed by _coalesce.  Row d writes at most cap entries starting at
 * d * cap; d_count[d] receives its entry count.  d_w_in is NULL or rows of
 * m-1 values with stride w_stride. */
int rg_conservative_1d(const double* d_xin, int64_t in_stride, int64_t m, const double* d_xout,
                       int64_t out_stride, int64_t n, int64_t nd, const double* d_w_in,
                       int64_t w_stride, int64_t cap, int64_t* d_ind_in, int64_t* d_ind_out,
                       double* d_val, int64_t* d_count, rg_stream_t stream);

/* Conservative transpose scaling of entries in the saved layout:
 * values * vol_in[i] / vol_out[o], first divided by w_in[i]^2 when d_w_in is
 * not NULL.  Replaces the loop of transpose_weights_conservative,
 * regridding/_weights/_weights_transposed/_weights_transposed.py:238-257.
 * Indices may be negative (counted from the end). */
int rg_transpose_conservative_scale(const int64_t* d_in, const int64_t* d_out, const double* d_val,
                                    int64_t nnz, const double* d_vol_in, int64_t n_in,
                                    const double* d_vol_out, int64_t n_out, const double* d_w_in,
                                    double* d_result, rg_stream_t stream);

/* Gradient of sum_{d,o} grad_out[d, o] * (W values)[d, o] with respect to the
 * output-grid vertex coordinates, for conservative 2D weights w built from
 * the given grids (the backward pass of a differentiable regrid; d_values and
 * d_grad_out are (stack, n_in) and (stack, n_out) of dtype RG_F32/RG_F64).
 * Writes d_grad_xo/d_grad_yo (nxo x nyo, zeroed first).  The derivative of
 * each overlap area comes from the overlap polygon of the output quad clipped
 * by the input quad, so input cells must be convex (RG_ERR_UNSUPPORTED
 * otherwise).  d_w_check, when not NULL, receives the weight of every stored
 * entry (CSR order) recomputed from that polygon.  Synchronises `stream`.
 * No upstream counterpart: the upstream weights have no derivative; this is
 * the adjoint of the overlap areas of
 * regridding/_weights/_weights_conservative_2d/_weights_conservative_2d.py:752-830. */
int rg_conservative_2d_grad_output(rg_weights w, const double* d_xi, const double* d_yi, int64_t nxi,
                                   int64_t nyi, const double* d_xo, const double* d_yo, int64_t nxo,
                                   int64_t nyo, const double* d_w_in, const void* d_values,
                                   const void* d_grad_out, int dtype, int64_t stack, double* d_grad_xo,
                                   double* d_grad_yo, double* d_w_check, rg_stream_t stream);

/* Linear (ny == 0) or bilinear interpolation of n_orth arrays at m index
 * points each: ndarray_linear_interpolation, regridding/_interp_ndarray.py
 * :11-268.  Array e has nx (x ny) float64 samples at d_a + e * a_stride and
 * its points' fractional indices at d_x (and d_y) + e * i_stride (a stride of
 * 0 shares one array or one set of points); d_out receives n_orth x m
 * float64 values.  Cells are floor(index) clamped to the first/last cell
 * (linear extrapolation outside), with the upstream operation order.
 * nx >= 2 and ny == 0 or ny >= 2 (RG_ERR_ARG otherwise). */
int rg_interp_linear(const double* d_a, int64_t a_stride, int64_t nx, int64_t ny, const double* d_x,
                     const double* d_y, int64_t i_stride, int64_t m, int64_t n_orth, double* d_out,
                     rg_stream_t stream);

/* fill(method="gauss_seidel"), regridding/_fill/_fill.py:10-109 and
 * _gauss_seidel.py:12-139, on a stack of nt slices of ny x nx cells
 * (C-ordered, dtype RG_F32/RG_F64) with the byte mask d_where (1 = missing),
 * in place: the missing cells are first set to the guess, then relaxed by
 * `iterations` red-black Gauss-Seidel iterations with periodic neighbours,
 * bit-identical to the upstream's sequential sweep (float32 arrays follow
 * Numba's typing: float32 neighbour sums, float64 products).  d_guess holds
 * one value per slice (RG_FILL_GUESS_SLICE) or per cell (RG_FILL_GUESS_FULL)
 * in the array's dtype; RG_FILL_GUESS_MEDIAN seeds with the per-slice median
 * of rg_fill_median.  An axis of length 1 with iterations > 0 is RG_ERR_ARG
 * (the upstream divides by zero). */
#define RG_FILL_GUESS_MEDIAN 0
#define RG_FILL_GUESS_SLICE 1
#define RG_FILL_GUESS_FULL 2
int rg_fill_gauss_seidel(void* d_a, int dtype, const uint8_t* d_where, int64_t nt, int64_t ny, int64_t nx,
                         const void* d_guess, int guess_kind, int64_t iterations, rg_stream_t stream);

/* The median of the valid (not missing, not NaN) cells of each of nt slices
 * of `slice` cells into d_out (nt values, the array's dtype), 0 for a slice
 * without valid cells: _guess_median, regridding/_fill/_gauss_seidel.py:61-80
 * (numpy's nanmedian: the mean of the two middle values for an even count). */
int rg_fill_median(const void* d_a, int dtype, const uint8_t* d_where, int64_t nt, int64_t slice, void* d_out,
                   rg_stream_t stream);

/* Device bytes currently held by a handle: the CSR plus whatever state
 * applies have made on first use (float32 weights, tile lists, transposed
 * CSR).  Used by caches that account weights against an HBM budget.  No
 * upstream counterpart. */
int rg_weights_device_bytes(rg_weights w, int64_t* bytes);

/* 64-bit hash of a host byte range (seeded), for cache keys of grids.  Host
 * code only; ranges above 4 MiB are hashed in 1 MiB segments on up to 8
 * host threads (the value does not depend on the thread count).  Not
 * cryptographic.  No upstream counterpart (the served form keys its weights
 * cache by grid hash). */
int rg_hash64(const void* h_data, int64_t nbytes, uint64_t seed, uint64_t* h_out);

/* rg_hash64 under two seeds in one pass over the bytes (inputs above 4 MiB
 * on up to 16 host threads): h_out[0] == rg_hash64(seed0), h_out[1] ==
 * rg_hash64(seed1) for inputs up to 4 MiB; above, the segment hashes of each
 * seed are combined as rg_hash64 combines them. */
int rg_hash64x2(const void* h_data, int64_t nbytes, uint64_t seed0, uint64_t seed1, uint64_t* h_out);

/* Copy nbytes from host memory (pageable or not) to the device on the
 * stream: on devices whose kernels access pageable host memory (Grace: ATS
 * over NVLink-C2C) by a kernel that reads the host array, so the copy does
 * not queue on the copy engines behind other streams' transfers; elsewhere
 * cudaMemcpyAsync.  Returns once the source has been read. */
int rg_copy_from_host(void* d_dst, const void* h_src, int64_t nbytes, rg_stream_t stream);

/* Attributes of the current device that choose the host-transfer strategy,
 * the first n of: SM count, asynchronous copy engines, pageable memory access
 * from kernels, whether that uses the host page tables, host pointers usable
 * for registered memory, concurrent managed access.  Host array of int64. */
int rg_device_attributes(int64_t* h_out, int n);

#ifdef __cplusplus
}
#endif

#endif /* REGRID_GB300_H */
