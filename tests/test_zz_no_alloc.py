"""The allocation-free locator, ``rg_locate_2d_noalloc``.

It exists for callers that cannot allocate device memory while they run: a
process whose GPU memory belongs to another allocator or a fixed budget, or a
latency-critical loop that must not meet an allocation's implicit
synchronisation or an out-of-memory error mid-stream.  Its scratch is a static
device array shared by every call, so these checks call it twice in a row and
compare each result with the allocating entry point, ``rg_locate_2d``
(method 2), which must agree exactly (cell indices are integers).
"""

import ctypes

import numpy as np
import pytest

import fixtures

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from regridding_gb300 import _lib

    return torch, _lib


def _locate(torch, lib_mod, fn, grid, px, py):
    x, y = (torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda() for a in grid)
    dpx = torch.from_numpy(np.ascontiguousarray(px, dtype=np.float64)).cuda()
    dpy = torch.from_numpy(np.ascontiguousarray(py, dtype=np.float64)).cuda()
    n = dpx.numel()
    oi = torch.full((n,), -7, dtype=torch.int64, device="cuda")
    oj = torch.full((n,), -7, dtype=torch.int64, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    P = ctypes.c_void_p
    args = [P(x.data_ptr()), P(y.data_ptr()), x.shape[0], x.shape[1], P(dpx.data_ptr()), P(dpy.data_ptr()), n]
    if fn == "rg_locate_2d":
        args.append(2)
    args += [P(oi.data_ptr()), P(oj.data_ptr()), s]
    lib_mod.call(fn, *args)
    torch.cuda.synchronize()
    return oi.cpu().numpy(), oj.cpu().numpy()


def test_noalloc_matches_allocating_locator_twice(env):
    torch, lib_mod = env
    g = fixtures.load("curvilinear.npz").case("curvi129").tuple("ci")
    rng = np.random.default_rng(11)
    for call in range(2):
        # points inside, outside (these go through the scratch list) and on vertices
        px = rng.uniform(-1.3, 1.3, 20000)
        py = rng.uniform(-1.3, 1.3, 20000)
        px[:64] = g[0][call + 3, 10:74]
        py[:64] = g[1][call + 3, 10:74]
        got = _locate(torch, lib_mod, "rg_locate_2d_noalloc", g, px, py)
        exp = _locate(torch, lib_mod, "rg_locate_2d", g, px, py)
        assert np.array_equal(got[0], exp[0]) and np.array_equal(got[1], exp[1]), f"call {call}"
        outside = got[0] == np.iinfo(np.int64).max
        assert outside.any() and (~outside).any()


def test_noalloc_rejects_oversized_calls(env):
    torch, lib_mod = env
    lib = lib_mod.load()
    limit = 1048576
    st = lib.rg_locate_2d_noalloc(None, None, 4, 4, None, None, limit + 1, None, None, None)
    assert st == lib_mod.RG_ERR_ARG
    assert "at most 1048576" in lib_mod.last_error()
