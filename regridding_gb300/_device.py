"""Device plumbing: torch CUDA buffers, the current stream, and device-resident weights.

torch is used only to own device memory and to name the CUDA stream; every
computation is a call into ``libregrid_gb300.so``.
"""

from __future__ import annotations

import concurrent.futures
import ctypes
import mmap
import os
import threading
import warnings
import weakref

import numpy as np

from . import _lib

_torch = None


def torch():
    """Import torch lazily and require a CUDA device (no CPU fallback)."""
    global _torch
    if _torch is None:
        import torch as t

        _torch = t
    if not _torch.cuda.is_available():
        raise _lib.RegridError("regridding_gb300 needs a CUDA device; none is available")
    return _torch


def stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch().cuda.current_stream().cuda_stream)


def ptr(t) -> ctypes.c_void_p | None:
    return None if t is None else ctypes.c_void_p(t.data_ptr())


# Arrays up to this size are uploaded by a kernel that reads the host array
# (rg_copy_from_host) where the device can read pageable host memory: grids
# and parameters then do not queue on the copy engines behind other streams'
# large transfers (120-190 GB/s from 8 MB up on GB300).
SM_UPLOAD_BYTES = 64 << 20
_host_access: dict[int, bool] = {}


def kernel_host_access() -> bool:
    """Whether kernels on the current device may read pageable host memory
    (asked once per device: the devices of one process can differ)."""
    dev = torch().cuda.current_device()
    v = _host_access.get(dev)
    if v is None:
        out = np.zeros(3, np.int64)
        _lib.call("rg_device_attributes", ctypes.c_void_p(out.ctypes.data), 3)
        v = _host_access[dev] = bool(out[2])
    return v


def _file_backed(a: np.ndarray) -> bool:
    """Whether the array's memory comes from a file mapping (np.memmap, the
    saved weights of store.load_weights): such pages may not be resident, and
    they are left to the copy engines rather than faulted in by a kernel."""
    b = a
    while b is not None:
        if isinstance(b, (np.memmap, mmap.mmap)):
            return True
        b = b.obj if isinstance(b, memoryview) else getattr(b, "base", None)
    return False


def upload(a: np.ndarray, dtype=None):
    """Host array -> contiguous CUDA tensor, copied straight from the
    array's (pageable) memory: on the Grace host of a GB300 a copy-engine
    copy runs at 110-160 GB/s for arrays of 8-34 MB, twice the rate of
    staging through a pinned copy first (whose host memcpy runs at 15-25
    GB/s); arrays up to SM_UPLOAD_BYTES go through a kernel instead (not
    file-mapped ones)."""
    t = torch()
    a = np.ascontiguousarray(a if dtype is None else np.asarray(a, dtype=dtype))
    if a.dtype == np.bool_:
        a = a.astype(np.uint8)
    if 0 < a.nbytes <= SM_UPLOAD_BYTES and kernel_host_access() and not _file_backed(a):
        d = t.empty(a.shape, dtype=t.from_numpy(np.empty(0, dtype=a.dtype)).dtype, device="cuda")
        _lib.call("rg_copy_from_host", ptr(d), ctypes.c_void_p(a.ctypes.data), a.nbytes, stream())
        return d
    with warnings.catch_warnings():
        # read-only arrays (the saved weights) are only read from
        warnings.simplefilter("ignore", UserWarning)
        host = t.from_numpy(a)
    return host.to("cuda")


def empty(shape, dtype):
    t = torch()
    return t.empty(shape, dtype=dtype, device="cuda")


# Large results go into a new host array whose pages are first touched by
# several threads: on the Grace host a device-to-host copy into untouched
# pageable memory runs at 14-25 GB/s (the copy takes every page fault on one
# thread), 16 threads touch 1.4 GB in ~6 ms, and the copy into touched
# memory then runs at ~190 GB/s.  Page-locked buffers would need a 80-150 ms
# allocation per 1.4 GB whenever the caller keeps the previous result.
PARALLEL_TOUCH_BYTES = 16 << 20
TOUCH_THREADS = min(16, os.cpu_count() or 1)
_touch_pool = None
_touch_lock = threading.Lock()


def _touch_pool_get():
    global _touch_pool
    with _touch_lock:
        if _touch_pool is None:
            _touch_pool = concurrent.futures.ThreadPoolExecutor(max_workers=TOUCH_THREADS,
                                                                thread_name_prefix="regrid-touch")
        return _touch_pool


def host_empty(shape, dtype) -> np.ndarray:
    """``numpy.empty`` with every page already faulted in (in parallel)."""
    a = np.empty(shape, dtype=dtype)
    if a.nbytes < PARALLEL_TOUCH_BYTES:
        return a
    b = a.reshape(-1).view(np.uint8)
    page = os.sysconf("SC_PAGE_SIZE") if hasattr(os, "sysconf") else 4096
    pool = _touch_pool_get()
    parts = TOUCH_THREADS
    edges = np.linspace(0, b.size // page, parts + 1).astype(np.int64) * page

    def touch(k):
        b[edges[k]:edges[k + 1]:page] = 0

    list(pool.map(touch, range(parts)))
    return a


def download(t) -> np.ndarray:
    t = t.detach()
    if t.is_cuda and t.numel() * t.element_size() >= PARALLEL_TOUCH_BYTES:
        a = host_empty(tuple(t.shape), np.dtype(str(t.dtype).replace("torch.", "")))
        torch().from_numpy(a).copy_(t)
        return a
    return t.cpu().numpy()


_TORCH_DTYPES = {}


def torch_dtype(np_dtype):
    t = torch()
    if not _TORCH_DTYPES:
        _TORCH_DTYPES.update({np.dtype(np.float32): t.float32, np.dtype(np.float64): t.float64,
                              np.dtype(np.int64): t.int64})
    return _TORCH_DTYPES[np.dtype(np_dtype)]


class DeviceWeights:
    """Sparse weights of one orthogonal element, resident in GPU memory.

    Rows are output cells and columns input cells.  Built by
    :func:`build_conservative_2d`, :meth:`from_coo` or the public
    :func:`regridding_gb300.weights`; applied with :meth:`apply`.
    """

    def __init__(self, handle: ctypes.c_void_p, shape_out: tuple[int, ...] | None = None,
                 shape_in: tuple[int, ...] | None = None):
        self._h = handle
        nnz, n_in, n_out = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.call("rg_weights_info", handle, ctypes.byref(nnz), ctypes.byref(n_in), ctypes.byref(n_out))
        self.nnz, self.n_in, self.n_out = nnz.value, n_in.value, n_out.value
        if shape_out is not None and len(shape_out) == 2 and shape_out[0] * shape_out[1] == self.n_out:
            _lib.call("rg_weights_set_output_shape", handle, int(shape_out[0]), int(shape_out[1]))
        if shape_in is not None and len(shape_in) == 2 and shape_in[0] * shape_in[1] == self.n_in:
            _lib.call("rg_weights_set_input_shape", handle, int(shape_in[0]), int(shape_in[1]))
        self._finalizer = weakref.finalize(self, _free_handle, handle.value)

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    @classmethod
    def from_coo(cls, indices_input, indices_output, values, n_in: int, n_out: int,
                 shape_out: tuple[int, ...] | None = None,
                 shape_in: tuple[int, ...] | None = None) -> "DeviceWeights":
        """Upload entries in the saved layout (numpy or CUDA tensors).  The
        2D shapes of the output and input cells, when given, let the fast
        apply tile rows and stage input boxes as for built weights."""
        t = torch()
        ii = _as_device(indices_input, t.int64)
        oo = _as_device(indices_output, t.int64)
        vv = _as_device(values, t.float64)
        h = ctypes.c_void_p()
        _lib.call("rg_weights_from_coo", ptr(ii), ptr(oo), ptr(vv), int(vv.numel()), int(n_in), int(n_out),
                  stream(), ctypes.byref(h))
        return cls(h, shape_out, shape_in)

    def export(self):
        """Entries in the saved layout, sorted by (input, output), as CUDA tensors."""
        t = torch()
        ii = t.empty(self.nnz, dtype=t.int64, device="cuda")
        oo = t.empty(self.nnz, dtype=t.int64, device="cuda")
        vv = t.empty(self.nnz, dtype=t.float64, device="cuda")
        _lib.call("rg_weights_export_coo", self._h, ptr(ii), ptr(oo), ptr(vv), stream())
        return ii, oo, vv

    def export_numpy(self):
        ii, oo, vv = self.export()
        return download(ii), download(oo), download(vv)

    def apply(self, values, out=None, accumulate: str = "exact", transpose: bool = False):
        """Apply to a CUDA tensor of shape (stack, n_in) (or (n_in,)).

        ``accumulate="exact"`` reproduces the upstream float64 result bit for
        bit (float64 output, or an upstream-style in-place float32 ``out``);
        ``"fast"`` accumulates in the output dtype with FMA; ``"compensated"``
        gives a float64 output within 1e-12 relative of the exact sum
        (float32 input: float-float arithmetic on the FP32 pipe; other dtypes
        compute as ``"exact"``).
        """
        t = torch()
        if accumulate not in _lib.RG_ACC:
            raise ValueError(f"accumulate must be one of {sorted(_lib.RG_ACC)}, got {accumulate!r}")
        n_src, n_dst = (self.n_out, self.n_in) if transpose else (self.n_in, self.n_out)
        squeeze = values.dim() == 1
        v = values.reshape(-1, n_src)
        if not v.is_contiguous():
            v = v.contiguous()
        if v.dtype not in (t.float32, t.float64):
            v = v.to(t.float64)
        stack = v.shape[0]
        if out is None:
            odt = v.dtype if accumulate == "fast" else t.float64
            out = t.empty((stack, n_dst), dtype=odt, device="cuda")
        o = out.reshape(stack, n_dst)
        acc = _lib.RG_ACC[accumulate]
        dt_in = _lib.RG_F32 if v.dtype == t.float32 else _lib.RG_F64
        dt_out = _lib.RG_F32 if o.dtype == t.float32 else _lib.RG_F64
        fn = "rg_apply_transpose" if transpose else "rg_apply"
        _lib.call(fn, self._h, ptr(v), dt_in, ptr(o), dt_out, int(stack), acc, stream())
        return out.reshape(n_dst) if squeeze and out.dim() == 2 else out

    def free(self) -> None:
        self._finalizer()


def _free_handle(h: int) -> None:
    try:
        lib = _lib.load(build_if_missing=False)
        s = None
        try:
            import torch as t

            if t.cuda.is_available():
                s = ctypes.c_void_p(t.cuda.current_stream().cuda_stream)
        except Exception:
            s = None
        lib.rg_weights_free(ctypes.c_void_p(h), s)
    except Exception:
        pass


def _as_device(a, dtype):
    t = torch()
    if isinstance(a, t.Tensor):
        return a.to(device="cuda", dtype=dtype).contiguous()
    return upload(np.asarray(a), dtype={t.int64: np.int64, t.float64: np.float64}[dtype])


def build_conservative_2d(grid_input, grid_output, weights_input=None) -> DeviceWeights:
    """Conservative weights of one element from (x, y) vertex grids (numpy or CUDA tensors)."""
    t = torch()
    xi, yi = (_as_device(a, t.float64) for a in grid_input)
    xo, yo = (_as_device(a, t.float64) for a in grid_output)
    nxi, nyi = xi.shape
    nxo, nyo = xo.shape
    wi = None if weights_input is None else _as_device(weights_input, t.float64)
    h = ctypes.c_void_p()
    _lib.call("rg_build_conservative_2d", ptr(xi), ptr(yi), nxi, nyi, ptr(xo), ptr(yo), nxo, nyo, ptr(wi),
              stream(), ctypes.byref(h))
    return DeviceWeights(h, (nxo - 1, nyo - 1))


def build_conservative_2d_batch(pairs, weights_input=None, max_cells: int = 48_000_000):
    """Conservative weights of many (grid_input, grid_output) pairs built
    together (``rg_build_conservative_2d_batch``): every stage of the build
    runs once over all pairs of a sub-batch.  Sub-batches hold at most
    ``max_cells`` input + output cells (the parallel walk's slot buffers scale
    with the cells of a sub-batch).  Returns one DeviceWeights per pair, or
    the RegridError of a pair whose build failed (degenerate grids), in
    order."""
    t = torch()
    n = len(pairs)
    if weights_input is None:
        weights_input = [None] * n
    dev = []
    for (gi, go), wi in zip(pairs, weights_input):
        xi, yi = (_as_device(a, t.float64) for a in gi)
        xo, yo = (_as_device(a, t.float64) for a in go)
        w = None if wi is None else _as_device(wi, t.float64)
        dev.append((xi, yi, xo, yo, w))
    results = [None] * n
    start = 0
    while start < n:
        stop, cells = start, 0
        while stop < n:
            xi, _, xo, _, _ = dev[stop]
            c = (xi.shape[0] - 1) * (xi.shape[1] - 1) + (xo.shape[0] - 1) * (xo.shape[1] - 1)
            if stop > start and cells + c > max_cells:
                break
            cells += c
            stop += 1
        m = stop - start
        P = ctypes.c_void_p * m
        I = ctypes.c_int64 * m
        part = dev[start:stop]
        xi_p = P(*(a[0].data_ptr() for a in part))
        yi_p = P(*(a[1].data_ptr() for a in part))
        xo_p = P(*(a[2].data_ptr() for a in part))
        yo_p = P(*(a[3].data_ptr() for a in part))
        wi_p = P(*((a[4].data_ptr() if a[4] is not None else None) for a in part))
        nxi = I(*(a[0].shape[0] for a in part))
        nyi = I(*(a[0].shape[1] for a in part))
        nxo = I(*(a[2].shape[0] for a in part))
        nyo = I(*(a[2].shape[1] for a in part))
        out = P()
        status = (ctypes.c_int * m)()
        _lib.call("rg_build_conservative_2d_batch", m, xi_p, yi_p, nxi, nyi, xo_p, yo_p, nxo, nyo,
                  wi_p if any(a[4] is not None for a in part) else None, stream(), out, status)
        for k in range(m):
            if status[k] == _lib.RG_OK:
                a = part[k]
                results[start + k] = DeviceWeights(ctypes.c_void_p(out[k]), (a[2].shape[0] - 1, a[2].shape[1] - 1))
            else:
                results[start + k] = _lib.RegridError(
                    f"conservative build of pair {start + k} failed (status {status[k]})")
        start = stop
    return results


# ---------------------------------------------------------------------------
# device-resident copies of saved weights, keyed by the identity of their
# numpy arrays; writable arrays (which the caller may have edited since)
# also by a hash of their contents
# ---------------------------------------------------------------------------

_cache_lock = threading.Lock()
_cache: dict[tuple, tuple] = {}


def content_hash(a: np.ndarray) -> tuple:
    """dtype, shape and two seeded 64-bit hashes of the array's bytes, taken
    in one pass on up to 16 host threads (rg_hash64x2)."""
    a = np.ascontiguousarray(a)
    h = (ctypes.c_uint64 * 2)()
    _lib.call("rg_hash64x2", ctypes.c_void_p(a.ctypes.data), a.nbytes, 0x5EED, 0xC0FFEE, h)
    return (a.dtype.str, a.shape, int(h[0]), int(h[1]))


def _fingerprint(element: tuple):
    """None for an element whose three arrays are read-only (the identity
    of the arrays is its key); else the content hashes of the three."""
    if all(not a.flags.writeable for a in element):
        return None
    return tuple(content_hash(a) for a in element)


def _drop(key: tuple) -> None:
    with _cache_lock:
        _cache.pop(key, None)


def remember(element: tuple, dw: DeviceWeights) -> None:
    """Associate the device copy with a saved-layout element (numpy arrays).
    Read-only arrays are recognised by identity; writable ones by identity
    and contents, so an element edited in place is uploaded again."""
    ii, oo, vv = element
    if not all(isinstance(a, np.ndarray) for a in (ii, oo, vv)):
        return
    key = (id(ii), id(oo), id(vv))
    fp = _fingerprint(element)
    with _cache_lock:
        _cache[key] = (weakref.ref(ii), weakref.ref(oo), weakref.ref(vv), dw, fp)
    weakref.finalize(vv, _drop, key)


def lookup(element: tuple, n_in: int, n_out: int) -> DeviceWeights | None:
    ii, oo, vv = element
    if not all(isinstance(a, np.ndarray) for a in (ii, oo, vv)):
        return None
    with _cache_lock:
        hit = _cache.get((id(ii), id(oo), id(vv)))
    if hit is None:
        return None
    ri, ro, rv, dw, fp = hit
    if ri() is not ii or ro() is not oo or rv() is not vv:
        return None
    if dw.n_in != n_in or dw.n_out != n_out:
        return None
    if fp is None:
        # remembered read-only: still read-only means unchanged
        return dw if all(not a.flags.writeable for a in element) else None
    return dw if _fingerprint(element) == fp else None
