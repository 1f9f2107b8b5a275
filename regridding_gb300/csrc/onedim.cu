// 1D kernels: find_indices (brute and searchsorted), multilinear weights and
// conservative 1D weights over batches of rows.
#include <cmath>

#include "common.cuh"

namespace rg {
namespace {

// numpy.searchsorted(a, v, side="left") on an ascending row: the first k with
// a[k] >= v in numpy's float order (NaN after every number).
__device__ __forceinline__ int64_t lower_bound_np(const double* a, int64_t n, double v) {
    int64_t lo = 0, hi = n;
    bool vnan = isnan(v);
    while (lo < hi) {
        int64_t mid = lo + ((hi - lo) >> 1);
        double am = __ldg(a + mid);
        bool lt = (am < v) || (vnan && !isnan(am));
        if (lt) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// _find_indices_searchsorted_1d post-processing: _find_indices_searchsorted.py:47-58
__device__ __forceinline__ int64_t searchsorted_cell(const double* a, int64_t m, double p,
                                                     int64_t fill) {
    int64_t r = lower_bound_np(a, m, p) - 1;
    if (p == __ldg(a)) r = 0;
    else if (r < 0) r = fill;
    else if (r > m - 2) r = fill;
    return r;
}

// Rows that are non-decreasing (and NaN free) answer the brute search with a
// binary search: for them the first m with a[m] <= p <= a[m+1] is exactly the
// searchsorted cell.  Other rows are scanned linearly.
__global__ void row_sorted_kernel(const double* x, int64_t stride, int64_t m, int64_t nrows,
                                  uint8_t* sorted) {
    int lane = threadIdx.x & 31;
    int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (r >= nrows) return;
    const double* a = x + r * stride;
    bool ok = true;
    for (int64_t k = lane; k + 1 < m; k += 32) ok &= (a[k] <= a[k + 1]);
    ok = __all_sync(0xffffffffu, ok);
    if (lane == 0) sorted[r] = ok;
}

__global__ void find_indices_kernel(const double* __restrict__ xin, int64_t in_stride, int64_t m,
                                    const double* __restrict__ xout, int64_t out_stride, int64_t n,
                                    int64_t nd, int method, int64_t fill,
                                    const uint8_t* __restrict__ sorted, int64_t* __restrict__ res) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nd * n;
         k += (int64_t)gridDim.x * blockDim.x) {
        int64_t d = k / n, i = k % n;
        const double* a = xin + d * in_stride;
        double p = xout[d * out_stride + i];
        int64_t r;
        if (method == 1) {
            r = searchsorted_cell(a, m, p, fill);
        } else if (m < 2) {
            r = fill;
        } else if (sorted[in_stride ? d : 0]) {
            r = searchsorted_cell(a, m, p, fill);
        } else {
            // _find_indices_brute_1d: _find_indices_brute.py:42-49
            r = fill;
            for (int64_t q = 0; q < m - 1; q++) {
                if (a[q] <= p && p <= a[q + 1]) {
                    r = q;
                    break;
                }
            }
        }
        res[k] = r;
    }
}

// _weights_from_indices_multilinear (_weights_multilinear.py:101-126) and
// _weights_from_indices_multilinear_1d (:169-202): raw entries 2i, 2i+1 of
// every row, plus the bucket (row, input index) and the in-bucket key
// (output index) used to put each row in the saved (input, output) order.
__global__ void multilinear_kernel(const double* __restrict__ xin, int64_t in_stride, int64_t m,
                                   const double* __restrict__ xout,
                                   const double* __restrict__ xsearch, int64_t out_stride, int64_t n,
                                   int64_t nd, const double* __restrict__ w_in, int64_t w_stride,
                                   int bounds, int32_t* __restrict__ bucket,
                                   int64_t* __restrict__ skey, double* __restrict__ raw_val,
                                   unsigned long long* __restrict__ n_outside) {
    const int64_t index_max = m - 2;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nd * n;
         k += (int64_t)gridDim.x * blockDim.x) {
        int64_t d = k / n, i = k % n;
        const double* a = xin + d * in_stride;
        double x = xout[d * out_stride + i];
        int64_t index = searchsorted_cell(a, m, xsearch ? xsearch[d * out_stride + i] : x, INT64_MAX);
        bool outside = (index < 0) || (index > index_max);
        if (outside && n_outside) atomicAdd(n_outside, 1ull);
        bool below = x < __ldg(a);
        int64_t i0 = below ? 0 : (index < 0 ? 0 : (index > index_max ? index_max : index));
        int64_t i1 = i0 + 1;
        double x0 = __ldg(a + i0), x1 = __ldg(a + i1);
        double w1 = ddiv(dsub(x, x0), dsub(x1, x0));
        double w0 = dsub(1.0, w1);
        if (w_in) {
            w0 = dmul(w0, w_in[d * w_stride + i0]);
            w1 = dmul(w1, w_in[d * w_stride + i1]);
        }
        if (bounds == RG_BOUNDS_NAN && outside) {
            w0 = NAN;
            w1 = NAN;
        }
        int64_t e = d * 2 * n + 2 * i;
        bucket[e] = (int32_t)(d * (m) + i0);
        bucket[e + 1] = (int32_t)(d * (m) + i1);
        skey[e] = i;
        skey[e + 1] = i;
        raw_val[e] = w0;
        raw_val[e + 1] = w1;
    }
}

__global__ void gather_multilinear(const uint32_t* __restrict__ perm, const int32_t* __restrict__ bucket,
                                   const int64_t* __restrict__ skey, const double* __restrict__ raw_val,
                                   int64_t total, int64_t m, int64_t* __restrict__ ind_in,
                                   int64_t* __restrict__ ind_out, double* __restrict__ val) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total;
         k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t e = perm[k];
        ind_in[k] = bucket[e] % m;
        ind_out[k] = skey[e];
        val[k] = raw_val[e];
    }
}

// One thread per row: _weights_conservative_1d
// (_weights_conservative_1d.py:59-318).  Grids are read through index maps
// instead of reversed copies.  Raw entries go to [d*cap, d*cap + count).
__global__ void conservative_1d_kernel(const double* __restrict__ xin, int64_t in_stride, int64_t m,
                                       const double* __restrict__ xout, int64_t out_stride,
                                       int64_t n, int64_t nd, const double* __restrict__ w_in,
                                       int64_t w_stride, int64_t cap, int64_t* __restrict__ ind_in,
                                       int64_t* __restrict__ ind_out, double* __restrict__ val,
                                       int64_t* __restrict__ count, unsigned* flags) {
    int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (d >= nd) return;
    const double* ai = xin + d * in_stride;
    const double* ao = xout + d * out_stride;
    const bool rev_in = !(ai[0] < ai[m - 1]);
    const bool rev_out = !(ao[0] < ao[n - 1]);
    auto xs = [&](int64_t k) { return rev_in ? ai[m - 1 - k] : ai[k]; };
    auto xt = [&](int64_t k) { return rev_out ? ao[n - 1 - k] : ao[k]; };
    // cell length of the (possibly reversed) sweep grid
    auto len_in = [&](int64_t k) { return dsub(xs(k + 1), xs(k)); };
    const double st_left = xt(0), st_right = xt(n - 1);
    int64_t base = d * cap, cnt = 0;
    int64_t isw = 0, ist;
    double p1 = xs(0);
    bool outside;
    if (st_left == p1) {
        outside = false;
        ist = 0;
    } else if (st_left < p1 && p1 < st_right) {
        outside = false;
        // index_of_point on the reversed-or-not static grid
        int64_t l = 0, r = n;
        while (r - l > 1) {
            int64_t mid = (l + r) / 2;
            if (xt(mid) > p1) r = mid;
            else l = mid;
        }
        ist = r - 1;
    } else {
        outside = true;
        ist = MAXSIZE;
    }
    while (isw < m - 1) {
        double p2 = xs(isw + 1);
        if (outside) {
            double ps = xt(0);
            if (p1 < ps && ps < p2) {
                ist = 0;
                p2 = ps;
            } else if (ps == p2) {
                isw = isw + 1;
                ist = 0;
            } else {
                isw = isw + 1;
            }
            if (ist < MAXSIZE) outside = false;
        } else {
            int64_t iin = isw, iout = ist;
            if (rev_in) iin = ~iin;
            if (rev_out) iout = ~iout;
            double ps = xt(ist + 1);
            if (p1 < ps && ps < p2) {
                ist = ist + 1;
                p2 = ps;
            } else if (ps == p2) {
                ist = ist + 1;
                isw = isw + 1;
            } else {
                isw = isw + 1;
            }
            double length = dsub(p2, p1);
            // negative indices wrap, as numpy indexing does
            int64_t li = iin < 0 ? iin + (m - 1) : iin;
            double ratio = ddiv(length, len_in(li));
            if (w_in) ratio = dmul(ratio, w_in[d * w_stride + li]);
            if (cnt >= cap) {
                atomicOr(flags, FLAG_CAPACITY);
                break;
            }
            ind_in[base + cnt] = iin;
            ind_out[base + cnt] = iout;
            val[base + cnt] = ratio;
            cnt++;
            if (!(0 <= ist && ist < n - 1)) break;
        }
        p1 = p2;
    }
    count[d] = cnt;
}

// Per-row keys for ordering conservative 1D entries by (input, output):
// negative (reversed-grid) indices are shifted by the row length, which keeps
// their order because a row's indices all have the same sign.
// Unused slots of a row (j >= count) are marked with PAD_INDEX and spread
// over the row's own buckets with keys that sort after every real entry, so
// no bucket grows long (the within-bucket ranking of long buckets is the
// expensive part of the sort); the merge skips them.
constexpr int64_t PAD_INDEX = INT64_MIN;

__global__ void conservative_1d_keys(int64_t* __restrict__ ind_in,
                                     const int64_t* __restrict__ ind_out,
                                     const int64_t* __restrict__ count, int64_t nd, int64_t cap,
                                     int64_t m, int64_t n, int32_t* __restrict__ bucket,
                                     int64_t* __restrict__ skey) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nd * cap;
         k += (int64_t)gridDim.x * blockDim.x) {
        int64_t d = k / cap, j = k % cap;
        if (j < count[d]) {
            int64_t i = ind_in[k];
            int64_t o = ind_out[k];
            if (i < 0) i += (m - 1);
            if (o < 0) o += (n - 1);
            bucket[k] = (int32_t)(d * (m - 1) + i);
            skey[k] = (o << 32) | (int64_t)j;
        } else {
            ind_in[k] = PAD_INDEX;
            bucket[k] = (int32_t)(d * (m - 1) + j % (m - 1));
            skey[k] = ((int64_t)INT32_MAX << 32) | (int64_t)j;
        }
    }
}

// Thread per row: gather the row's sorted entries and merge equal pairs
// (add.reduceat association; pairs are unique in practice).
__global__ void conservative_1d_merge(const uint32_t* __restrict__ perm, const int64_t* __restrict__ bptr,
                                      const int64_t* __restrict__ in_raw,
                                      const int64_t* __restrict__ out_raw,
                                      const double* __restrict__ val_raw, int64_t nd, int64_t m,
                                      int64_t cap, int64_t* __restrict__ ind_in,
                                      int64_t* __restrict__ ind_out, double* __restrict__ val,
                                      int64_t* __restrict__ count) {
    int64_t d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (d >= nd) return;
    int64_t s = bptr[d * (m - 1)], t = bptr[(d + 1) * (m - 1)];
    int64_t w = 0;
    int64_t g = s;
    while (g < t) {
        uint32_t e = perm[g];
        int64_t ii = in_raw[e], oo = out_raw[e];
        if (ii == PAD_INDEX) {  // unused slot (sorted last in its bucket)
            g++;
            continue;
        }
        double acc = val_raw[e];
        // group of equal pairs: first + (sequential from -0.0 over the rest,
        // exact for the < 8 extra terms a 1D overlap can produce)
        int64_t h = g + 1;
        double rest = -0.0;
        while (h < t && in_raw[perm[h]] == ii && out_raw[perm[h]] == oo) {
            rest = dadd(rest, val_raw[perm[h]]);
            h++;
        }
        if (h - g > 1) acc = dadd(acc, rest);
        ind_in[d * cap + w] = ii;
        ind_out[d * cap + w] = oo;
        val[d * cap + w] = acc;
        w++;
        g = h;
    }
    count[d] = w;
}

__global__ void cell_length_kernel(const double* x, int64_t nd, int64_t n, double* len) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nd * (n - 1);
         k += (int64_t)gridDim.x * blockDim.x) {
        int64_t d = k / (n - 1), i = k % (n - 1);
        len[k] = dsub(x[d * n + i + 1], x[d * n + i]);
    }
}

__global__ void transpose_scale_kernel(const int64_t* __restrict__ ii, const int64_t* __restrict__ oo,
                                       const double* __restrict__ v, int64_t nnz,
                                       const double* __restrict__ vol_in, int64_t n_in,
                                       const double* __restrict__ vol_out, int64_t n_out,
                                       const double* __restrict__ w_in, double* __restrict__ res) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz;
         k += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = ii[k] < 0 ? ii[k] + n_in : ii[k];
        int64_t o = oo[k] < 0 ? oo[k] + n_out : oo[k];
        if (i < 0 || i >= n_in || o < 0 || o >= n_out) {
            res[k] = NAN;  // index outside the grids: no volume to scale by
            continue;
        }
        double x = v[k];
        if (w_in) {
            double wi = w_in[i];
            x = ddiv(x, dmul(wi, wi));
        }
        res[k] = ddiv(dmul(x, vol_in[i]), vol_out[o]);
    }
}

}  // namespace

int find_indices_1d(const double* xin, int64_t in_stride, int64_t m, const double* xout,
                    int64_t out_stride, int64_t n, int64_t nd, int method, int64_t fill,
                    int64_t* res, cudaStream_t s) {
    RG_CHECK(method == 0 || method == 1, RG_ERR_ARG, "find_indices: unknown method %d", method);
    if (nd * n <= 0) return RG_OK;
    RG_CHECK(m >= 1, RG_ERR_ARG, "find_indices: empty input grid");
    uint8_t* sorted = nullptr;
    int64_t nrows = in_stride ? nd : 1;
    if (method == 0) {
        RG_TRY(dalloc(&sorted, (size_t)nrows, s));
        row_sorted_kernel<<<grid_for(nrows * 32, 256), 256, 0, s>>>(xin, in_stride, m, nrows, sorted);
    }
    unsigned g = grid_for(nd * n, 256);
    if (g > 65536) g = 65536;
    find_indices_kernel<<<g, 256, 0, s>>>(xin, in_stride, m, xout, out_stride, n, nd, method, fill,
                                          sorted, res);
    dfree(sorted, s);
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

int multilinear_1d(const double* xin, int64_t in_stride, int64_t m, const double* xout,
                   const double* xsearch, int64_t out_stride, int64_t n, int64_t nd, const double* w_in,
                   int64_t w_stride,
                   int bounds, int64_t* ind_in, int64_t* ind_out, double* val, int64_t* h_n_outside,
                   cudaStream_t s) {
    RG_CHECK(m >= 2, RG_ERR_ARG, "multilinear: the input grid needs at least 2 vertices");
    RG_CHECK(bounds >= 0 && bounds <= 2, RG_ERR_ARG, "multilinear: unknown bounds %d", bounds);
    int64_t total = 2 * n * nd;
    if (total == 0) return RG_OK;
    RG_CHECK(nd * m < INT32_MAX, RG_ERR_UNSUPPORTED,
             "multilinear: rows x input vertices must stay below 2^31");
    int32_t* bucket = nullptr;
    int64_t* skey = nullptr;
    double* raw_val = nullptr;
    int64_t* bptr = nullptr;
    uint32_t* perm = nullptr;
    unsigned long long* nout = nullptr;
    int st = RG_OK;
    do {
        if ((st = dalloc(&bucket, (size_t)total, s))) break;
        if ((st = dalloc(&skey, (size_t)total, s))) break;
        if ((st = dalloc(&raw_val, (size_t)total, s))) break;
        if ((st = dalloc(&nout, 1, s))) break;
        cudaMemsetAsync(nout, 0, sizeof(unsigned long long), s);
        unsigned g = grid_for(nd * n, 256);
        if (g > 65536) g = 65536;
        multilinear_kernel<<<g, 256, 0, s>>>(xin, in_stride, m, xout, xsearch, out_stride, n, nd, w_in, w_stride,
                                             bounds, bucket, skey, raw_val, nout);
        if (bounds == RG_BOUNDS_RAISE || h_n_outside) {
            unsigned long long h = 0;
            cudaMemcpyAsync(&h, nout, sizeof(h), cudaMemcpyDeviceToHost, s);
            cudaError_t e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) {
                set_error("multilinear: %s", cudaGetErrorString(e));
                st = RG_ERR_CUDA;
                break;
            }
            if (h_n_outside) *h_n_outside = (int64_t)h;
            if (bounds == RG_BOUNDS_RAISE && h) break;
        }
        if ((st = dalloc(&bptr, (size_t)(nd * m) + 1, s))) break;
        if ((st = dalloc(&perm, (size_t)total, s))) break;
        if ((st = bucket_sort(bucket, skey, total, nd * m, bptr, perm, nullptr, s))) break;
        g = grid_for(total, 256);
        if (g > 65536) g = 65536;
        gather_multilinear<<<g, 256, 0, s>>>(perm, bucket, skey, raw_val, total, m, ind_in, ind_out, val);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error("multilinear: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
        }
    } while (0);
    dfree(bucket, s);
    dfree(skey, s);
    dfree(raw_val, s);
    dfree(bptr, s);
    dfree(perm, s);
    dfree(nout, s);
    return st;
}

int conservative_1d(const double* xin, int64_t in_stride, int64_t m, const double* xout,
                    int64_t out_stride, int64_t n, int64_t nd, const double* w_in, int64_t w_stride,
                    int64_t cap, int64_t* ind_in, int64_t* ind_out, double* val, int64_t* count,
                    cudaStream_t s) {
    RG_CHECK(m >= 2 && n >= 2, RG_ERR_ARG, "conservative 1D: grids need at least 2 vertices");
    if (nd <= 0) return RG_OK;
    RG_CHECK(nd * (m - 1) < INT32_MAX && nd * cap < UINT32_MAX, RG_ERR_UNSUPPORTED,
             "conservative 1D: batch too large");
    int64_t total = nd * cap;
    int64_t *r_in = nullptr, *r_out = nullptr, *skey = nullptr, *bptr = nullptr;
    double* r_val = nullptr;
    int32_t* bucket = nullptr;
    uint32_t* perm = nullptr;
    unsigned* flags = nullptr;
    int st = RG_OK;
    do {
        if ((st = dalloc(&r_in, (size_t)total, s))) break;
        if ((st = dalloc(&r_out, (size_t)total, s))) break;
        if ((st = dalloc(&r_val, (size_t)total, s))) break;
        if ((st = dalloc(&flags, 1, s))) break;
        cudaMemsetAsync(flags, 0, sizeof(unsigned), s);
        conservative_1d_kernel<<<grid_for(nd, 128), 128, 0, s>>>(xin, in_stride, m, xout, out_stride, n, nd,
                                                                 w_in, w_stride, cap, r_in, r_out, r_val,
                                                                 count, flags);
        if ((st = dalloc(&bucket, (size_t)total, s))) break;
        if ((st = dalloc(&skey, (size_t)total, s))) break;
        unsigned g = grid_for(total, 256);
        if (g > 65536) g = 65536;
        conservative_1d_keys<<<g, 256, 0, s>>>(r_in, r_out, count, nd, cap, m, n, bucket, skey);
        int64_t nb = nd * (m - 1);
        if ((st = dalloc(&bptr, (size_t)nb + 1, s))) break;
        if ((st = dalloc(&perm, (size_t)total, s))) break;
        if ((st = bucket_sort(bucket, skey, total, nb, bptr, perm, nullptr, s))) break;
        conservative_1d_merge<<<grid_for(nd, 128), 128, 0, s>>>(perm, bptr, r_in, r_out, r_val, nd, m, cap,
                                                                ind_in, ind_out, val, count);
        unsigned fl = 0;
        cudaMemcpyAsync(&fl, flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("conservative 1D: %s", cudaGetErrorString(e));
            st = RG_ERR_CUDA;
            break;
        }
        if (fl & FLAG_CAPACITY) {
            set_error("conservative 1D: per-row capacity %lld exceeded", (long long)cap);
            st = RG_ERR_ARG;
        }
    } while (0);
    dfree(r_in, s);
    dfree(r_out, s);
    dfree(r_val, s);
    dfree(skey, s);
    dfree(bptr, s);
    dfree(bucket, s);
    dfree(perm, s);
    dfree(flags, s);
    return st;
}

int cell_length_1d(const double* x, int64_t nd, int64_t n, double* len, cudaStream_t s) {
    if (nd * (n - 1) <= 0) return RG_OK;
    unsigned g = grid_for(nd * (n - 1), 256);
    if (g > 65536) g = 65536;
    cell_length_kernel<<<g, 256, 0, s>>>(x, nd, n, len);
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

int transpose_conservative_scale(const int64_t* ii, const int64_t* oo, const double* v, int64_t nnz,
                                 const double* vol_in, int64_t n_in, const double* vol_out,
                                 int64_t n_out, const double* w_in, double* res, cudaStream_t s) {
    if (nnz <= 0) return RG_OK;
    unsigned g = grid_for(nnz, 256);
    if (g > 65536) g = 65536;
    transpose_scale_kernel<<<g, 256, 0, s>>>(ii, oo, v, nnz, vol_in, n_in, vol_out, n_out, w_in, res);
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

namespace {

// ndarray_linear_interpolation (regridding/_interp_ndarray.py:166-268): one
// thread per output point; element e of the orthogonal batch reads its
// samples at a + e * a_stride (stride 0: one array for all elements) and its
// indices at x + e * i_stride (likewise).  The cell is floor(x) moved into
// [0, n - 2] (linear extrapolation outside, :208-213), and the point formulas
// keep the upstream operation order with one rounding per operation.  The
// host guarantees n >= 2 on every interpolated axis, so all four reads stay
// inside the array; floor() of a huge or NaN index converts with saturation
// and is then clamped like any other.
__device__ __forceinline__ int64_t interp_cell(double v, int64_t n) {
    int64_t c = (int64_t)floor(v);
    if (c < 0) c = 0;
    else if (c > n - 2) c = n - 2;
    return c;
}

// The per-point part of the upstream formulas: the cell and the weights
// (1D: w00 = 1 - dx, w10 = dx).  When every element shares the points it is
// computed once per point and reused for all the elements a thread visits,
// which halves the FP64 operations per output value (the FP64 pipe, not HBM,
// bounds this kernel on GB300).
struct InterpPoint {
    int64_t i0, j0;
    double w00, w01, w10, w11;
};

__device__ __forceinline__ InterpPoint interp_point(double xv, double yv, int64_t nx, int64_t ny) {
    InterpPoint q;
    q.i0 = interp_cell(xv, nx);
    const double dx = dsub(xv, (double)q.i0);
    if (ny == 0) {
        q.j0 = 0;
        q.w00 = dsub(1.0, dx);
        q.w10 = dx;
        q.w01 = q.w11 = 0.0;
    } else {
        q.j0 = interp_cell(yv, ny);
        const double dy = dsub(yv, (double)q.j0);
        q.w00 = dmul(dsub(1.0, dx), dsub(1.0, dy));
        q.w01 = dmul(dsub(1.0, dx), dy);
        q.w10 = dmul(dx, dsub(1.0, dy));
        q.w11 = dmul(dx, dy);
    }
    return q;
}

// a0 * (1 - dx) + a1 * dx (:217), and (a00 * w00) + (a01 * w01) + (a10 * w10)
// + (a11 * w11) left to right (:268).
__device__ __forceinline__ double interp_eval(const double* __restrict__ s, const InterpPoint& q, int64_t ny) {
    if (ny == 0) return dadd(dmul(s[q.i0], q.w00), dmul(s[q.i0 + 1], q.w10));
    const double* r0 = s + q.i0 * ny + q.j0;
    const double* r1 = r0 + ny;
    return dadd(dadd(dadd(dmul(r0[0], q.w00), dmul(r0[1], q.w01)), dmul(r1[0], q.w10)), dmul(r1[1], q.w11));
}

// Thread = one point p for a run of `run` consecutive elements (grid y);
// reads of each element's samples by neighbouring threads fall on
// neighbouring points, and the output rows are written coalesced.
__global__ void interp_kernel(const double* __restrict__ a, int64_t a_stride, int64_t nx, int64_t ny,
                              const double* __restrict__ x, const double* __restrict__ y, int64_t i_stride,
                              int64_t m, int64_t n_orth, int64_t run, double* __restrict__ out) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < m; p += (int64_t)gridDim.x * blockDim.x) {
        for (int64_t e0 = blockIdx.y * run; e0 < n_orth; e0 += (int64_t)gridDim.y * run) {
            const int64_t e1 = e0 + run < n_orth ? e0 + run : n_orth;
            if (i_stride == 0) {
                const InterpPoint q = interp_point(x[p], ny ? y[p] : 0.0, nx, ny);
                for (int64_t e = e0; e < e1; ++e) out[e * m + p] = interp_eval(a + e * a_stride, q, ny);
            } else {
                for (int64_t e = e0; e < e1; ++e) {
                    const int64_t k = e * i_stride + p;
                    const InterpPoint q = interp_point(x[k], ny ? y[k] : 0.0, nx, ny);
                    out[e * m + p] = interp_eval(a + e * a_stride, q, ny);
                }
            }
        }
    }
}

}  // namespace

}  // namespace rg

extern "C" int rg_interp_linear(const double* d_a, int64_t a_stride, int64_t nx, int64_t ny, const double* d_x,
                                const double* d_y, int64_t i_stride, int64_t m, int64_t n_orth, double* d_out,
                                rg_stream_t stream) {
    rg::NvtxRange nvtx_range("rg_interp_linear");
    using namespace rg;
    RG_CHECK(nx >= 2 && (ny == 0 || ny >= 2) && m >= 0 && n_orth >= 0 && a_stride >= 0 && i_stride >= 0, RG_ERR_ARG,
             "rg_interp_linear: every interpolated axis needs at least 2 samples");
    RG_CHECK(ny == 0 || d_y, RG_ERR_ARG, "rg_interp_linear: 2D interpolation needs y indices");
    if (m == 0 || n_orth == 0) return RG_OK;
    RG_CHECK(d_a && d_x && d_out, RG_ERR_ARG, "rg_interp_linear: NULL argument");
    const int64_t run = i_stride == 0 ? (n_orth < 16 ? n_orth : 16) : 1;
    const int64_t runs = (n_orth + run - 1) / run;
    const unsigned gx = grid_for(m, 256) > (1u << 20) ? (1u << 20) : grid_for(m, 256);
    const unsigned gy = runs > 65535 ? 65535u : (unsigned)runs;
    interp_kernel<<<dim3(gx, gy), 256, 0, (cudaStream_t)stream>>>(d_a, a_stride, nx, ny, d_x, d_y, i_stride, m,
                                                                  n_orth, run, d_out);
    RG_CUDA(cudaGetLastError());
    return RG_OK;
}

