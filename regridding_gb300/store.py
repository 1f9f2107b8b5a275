"""On-disk weights: a memory-mappable file format for the saved layout and a
directory cache of built weights keyed by grid hash.

The upstream saves weights as ``(array, shape_input, shape_output)`` where
each element of ``array`` is ``(indices_input int64, indices_output int64,
values float64)`` and describes "a form [that] pickles and memory-maps
cleanly" (regridding/_weights/_weights.py:31-36).  It leaves storage to the
caller.  This module gives that form a file:

* :func:`save_weights` / :func:`load_weights` — one file per saved layout:
  a 64-byte preamble (magic, header length), a JSON header (element shape,
  ``shape_input``, ``shape_output``, entry count, byte offsets) and four
  arrays, each starting on a 4096-byte boundary: per-element entry offsets
  (int64, ``n_elements + 1``) and the concatenated ``indices_input``,
  ``indices_output`` and ``values`` of all elements.  :func:`load_weights`
  maps the file and returns the saved layout whose elements are read-only
  views of the mapping, so a load costs no copy and weights larger than
  host memory page in on use.  Read-only elements are also what the
  device-copy cache of :func:`regridding_gb300.regrid_from_weights` keys on,
  so a loaded layout is uploaded to the GPU once per process.
* :class:`WeightsDiskCache` — a directory of such files named by the hash of
  everything the weights depend on (coordinate arrays, axes,
  ``weights_input``, method, bounds, perturbation and seed; the coordinate
  hashes are the serving cache's :func:`~regridding_gb300.serving.grid_key`)
  and of the build that makes them (:func:`build_tag`: library version and
  weights revision, also stored in every file's header and checked on a
  hit).  A short or corrupt file reads as a miss.
  :meth:`WeightsDiskCache.weights` has the signature of
  :func:`regridding_gb300.weights` and returns the stored layout on a hit,
  else builds, stores and returns it.  Files are written to a temporary name
  and renamed into place, so concurrent processes sharing the directory
  never read a partial file; the least recently used files are removed
  beyond ``max_bytes``.
"""

from __future__ import annotations

import hashlib
import json
import os
import tempfile
import threading
from typing import Sequence

import numpy as np

from . import _util

__all__ = ["save_weights", "load_weights", "WeightsDiskCache", "weights_key"]

MAGIC = b"RGWEIGHTS1\0\0\0\0\0\0"
PREAMBLE = 64
ALIGN = 4096
WEIGHTS_REVISION = 2
"""Raised whenever the weights this library builds from the same arguments
may change (an arithmetic or layout change of the build); with the
library version it names the build that wrote a cache file."""


def build_tag() -> str:
    """The library version and weights revision: part of every cache key and
    of every file's header, so a cache never serves weights of another build."""
    from . import _lib

    return f"rg{int(_lib.load().rg_version())}-w{WEIGHTS_REVISION}"


def _align(n: int) -> int:
    return (n + ALIGN - 1) // ALIGN * ALIGN


def _elements(array) -> list:
    flat = np.asarray(array, dtype=object).reshape(-1)
    out = []
    for k in range(flat.size):
        ii, oo, vv = flat[k]
        out.append((np.asarray(ii, dtype=np.int64).reshape(-1), np.asarray(oo, dtype=np.int64).reshape(-1),
                    np.asarray(vv, dtype=np.float64).reshape(-1)))
    return out


def save_weights(path, weights, meta: dict | None = None) -> int:
    """Write the saved layout ``(array, shape_input, shape_output)`` to
    ``path`` (atomically: a temporary file renamed into place); returns the
    file size in bytes.  ``meta`` (JSON-serialisable) is kept in the
    header."""
    array, shape_input, shape_output = weights
    shape = tuple(int(s) for s in np.shape(array))
    elems = _elements(array)
    counts = np.array([len(e[2]) for e in elems], dtype=np.int64)
    for ii, oo, vv in elems:
        if not (len(ii) == len(oo) == len(vv)):
            raise ValueError("every element needs indices_input, indices_output and values of one length")
    offsets = np.zeros(len(elems) + 1, dtype=np.int64)
    np.cumsum(counts, out=offsets[1:])
    total = int(offsets[-1])
    header = {
        "format": 1,
        "shape": list(shape),
        "shape_input": [int(s) for s in shape_input],
        "shape_output": [int(s) for s in shape_output],
        "entries": total,
        "build": build_tag(),
        "meta": meta or {},
    }
    # layout: preamble | header | offsets | indices_input | indices_output | values
    sizes = [offsets.nbytes, 8 * total, 8 * total, 8 * total]
    raw = json.dumps(header).encode()
    pos = _align(PREAMBLE + len(raw) + 256)  # room for the offsets written below
    starts = []
    for n in sizes:
        starts.append(pos)
        pos = _align(pos + n)
    header["offsets"] = starts
    raw = json.dumps(header).encode()
    if PREAMBLE + len(raw) > starts[0]:
        raise ValueError("header too long")  # never: 256 bytes cover four offsets
    directory = os.path.dirname(os.path.abspath(path))
    fd, tmp = tempfile.mkstemp(prefix=".rgw-", dir=directory)
    try:
        with os.fdopen(fd, "wb") as f:
            f.write(MAGIC + len(raw).to_bytes(8, "little") + bytes(PREAMBLE - len(MAGIC) - 8))
            f.write(raw)
            f.seek(starts[0])
            f.write(offsets.tobytes())
            for col, start in zip(range(3), starts[1:]):
                f.seek(start)
                for e in elems:
                    f.write(np.ascontiguousarray(e[col]).tobytes())
            f.truncate(pos)
        os.replace(tmp, path)
    except BaseException:
        try:
            os.unlink(tmp)
        except OSError:
            pass
        raise
    return pos


def read_header(path) -> dict:
    """The JSON header of a weights file."""
    with open(path, "rb") as f:
        pre = f.read(PREAMBLE)
        if len(pre) < PREAMBLE or pre[: len(MAGIC)] != MAGIC:
            raise ValueError(f"{path} is not a weights file")
        n = int.from_bytes(pre[len(MAGIC): len(MAGIC) + 8], "little")
        return json.loads(f.read(n))


def load_weights(path, mmap: bool = True):
    """The saved layout ``(array, shape_input, shape_output)`` stored in
    ``path``.  With ``mmap`` the element arrays are read-only views of a
    memory mapping of the file; otherwise they are read into memory (and
    are still read-only)."""
    header = read_header(path)
    try:
        total = int(header["entries"])
        n_elem = int(np.prod(header["shape"], dtype=np.int64))
        s_off, s_in, s_out, s_val = (int(v) for v in header["offsets"])
    except (KeyError, TypeError, ValueError) as exc:
        raise ValueError(f"{path}: malformed header ({exc})") from None
    size = os.path.getsize(path)
    ends = (s_off + 8 * (n_elem + 1), s_in + 8 * total, s_out + 8 * total, s_val + 8 * total)
    if total < 0 or n_elem < 0 or min(s_off, s_in, s_out, s_val) < PREAMBLE or max(ends) > size:
        raise ValueError(f"{path}: truncated or corrupt (arrays end past the file's {size} bytes)")
    if mmap:
        mm = np.memmap(path, dtype=np.uint8, mode="r")

        def view(start, count, dtype):
            return mm[start: start + count * 8].view(dtype)
    else:
        with open(path, "rb") as f:
            blob = np.frombuffer(f.read(), dtype=np.uint8)

        def view(start, count, dtype):
            return blob[start: start + count * 8].view(dtype)

    offsets = view(s_off, n_elem + 1, np.int64)
    if offsets[0] != 0 or offsets[-1] != total or np.any(np.diff(offsets) < 0):
        raise ValueError(f"{path}: corrupt element offsets")
    ii, oo, vv = view(s_in, total, np.int64), view(s_out, total, np.int64), view(s_val, total, np.float64)
    flat = np.empty(n_elem, dtype=object)
    for k in range(n_elem):
        a, b = int(offsets[k]), int(offsets[k + 1])
        flat[k] = (ii[a:b], oo[a:b], vv[a:b])
    array = flat.reshape(tuple(header["shape"]))
    return array, tuple(header["shape_input"]), tuple(header["shape_output"])


def _array_digest(a) -> list:
    from .serving import _hash_array

    a = np.asarray(a)
    dt, shape, h1, h2 = _hash_array(a)
    return [dt, list(shape), h1, h2]


def weights_key(coordinates_input, coordinates_output, axis_input=None, axis_output=None, weights_input=None,
                method: str = "multilinear", bounds: str = "extrapolate", perturb=None,
                seed=_util.SEED_DEFAULT, grids: tuple | None = None) -> str | None:
    """Hex digest naming the weights of one :func:`regridding_gb300.weights`
    call, or None when the call is not reproducible from its arguments (a
    ``numpy.random.Generator`` seed, whose state changes with use).
    ``grids`` is the coordinates' :func:`~regridding_gb300.serving.grid_key`
    when the caller already has it.  Arguments without effect on the result
    are left out (``perturb=None`` is resolved as ``weights`` resolves it,
    the seed counts only when perturbing, the bounds only for multilinear
    weights), so equivalent calls share a key."""
    if isinstance(seed, np.random.Generator):
        return None
    from .serving import grid_key

    ci = coordinates_input if isinstance(coordinates_input, tuple) else (coordinates_input,)
    co = coordinates_output if isinstance(coordinates_output, tuple) else (coordinates_output,)
    if grids is None:
        grids = grid_key(ci, co)
    if perturb is None:
        perturb = method == "conservative" and len(ci) >= 2
    parts = {
        "grids": [[dt, list(shape), int(h1), int(h2)] for dt, shape, h1, h2 in grids],
        "n_input": len(ci),
        "axis_input": None if axis_input is None else np.atleast_1d(axis_input).tolist(),
        "axis_output": None if axis_output is None else np.atleast_1d(axis_output).tolist(),
        "weights_input": None if weights_input is None else _array_digest(weights_input),
        "method": method,
        "bounds": bounds if method == "multilinear" else None,
        "perturb": bool(perturb),
        "seed": None if (seed is None or not perturb) else int(seed),
        "build": build_tag(),
    }
    return hashlib.sha256(json.dumps(parts, sort_keys=True).encode()).hexdigest()[:40]


class WeightsDiskCache:
    """A directory of weights files keyed by :func:`weights_key`."""

    SUFFIX = ".rgw"

    def __init__(self, directory, max_bytes: float | None = None):
        self.directory = os.fspath(directory)
        os.makedirs(self.directory, exist_ok=True)
        self.max_bytes = None if max_bytes is None else int(max_bytes)
        self._lock = threading.Lock()
        self.hits = self.misses = self.writes = self.evictions = 0

    def path(self, key: str) -> str:
        return os.path.join(self.directory, key + self.SUFFIX)

    def get(self, key: str | None, mmap: bool = True):
        """The stored layout of ``key`` (a hit refreshes its recency), or None."""
        if key is None:
            return None
        p = self.path(key)
        try:
            if read_header(p).get("build") != build_tag():
                raise ValueError("written by another build")
            w = load_weights(p, mmap=mmap)
        except (FileNotFoundError, ValueError, json.JSONDecodeError):
            with self._lock:
                self.misses += 1
            return None
        try:
            os.utime(p)
        except OSError:
            pass
        with self._lock:
            self.hits += 1
        return w

    def put(self, key: str | None, weights, meta: dict | None = None) -> None:
        if key is None:
            return
        save_weights(self.path(key), weights, meta)
        with self._lock:
            self.writes += 1
        self.trim()

    def entries(self) -> list[tuple[float, int, str]]:
        """(last use, size, path) of every stored file, oldest first."""
        out = []
        for name in os.listdir(self.directory):
            if name.endswith(self.SUFFIX):
                p = os.path.join(self.directory, name)
                try:
                    st = os.stat(p)
                except FileNotFoundError:
                    continue
                out.append((st.st_mtime, st.st_size, p))
        return sorted(out)

    def nbytes(self) -> int:
        return sum(e[1] for e in self.entries())

    def trim(self) -> None:
        """Remove the least recently used files beyond ``max_bytes``."""
        if self.max_bytes is None:
            return
        entries = self.entries()
        total = sum(e[1] for e in entries)
        for _, size, p in entries:
            if total <= self.max_bytes:
                break
            try:
                os.unlink(p)
            except FileNotFoundError:
                pass
            total -= size
            with self._lock:
                self.evictions += 1

    def weights(
        self,
        coordinates_input: tuple[np.ndarray, ...],
        coordinates_output: tuple[np.ndarray, ...],
        axis_input: None | int | Sequence[int] = None,
        axis_output: None | int | Sequence[int] = None,
        weights_input: None | np.ndarray = None,
        method: str = "multilinear",
        bounds: str = "extrapolate",
        perturb: None | bool = None,
        seed=_util.SEED_DEFAULT,
    ):
        """:func:`regridding_gb300.weights` through the cache."""
        from ._weights import weights as build

        key = weights_key(coordinates_input, coordinates_output, axis_input, axis_output, weights_input, method,
                          bounds, perturb, seed)
        hit = self.get(key)
        if hit is not None:
            return hit
        w = build(coordinates_input, coordinates_output, axis_input=axis_input, axis_output=axis_output,
                  weights_input=weights_input, method=method, bounds=bounds, perturb=perturb, seed=seed)
        if key is not None:
            self.put(key, w, {"method": method})
            stored = self.get(key)
            if stored is not None:
                with self._lock:
                    self.hits -= 1  # the read-back of a fresh build is not a hit
                return stored
        return w
