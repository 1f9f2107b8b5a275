"""Failure paths of the build, exercised on the GPU without a GPU fault.

* An undersized triple buffer: RG_FAULT_CHUNK_SLOTS caps the slots each
  chunk of the parallel walk gets, so chunks overflow their buffers (the
  device flags it; nothing is written past a buffer) and the build takes its
  recovery path, whole-line walks sized by an exact count.  The weights are
  bit-identical to the normal build's and to the oracle's.
* The debug library (RG_DEBUG=1: bounds-checked grid reads in the builds,
  an out-of-range read recorded as an error status rather than a trap)
  builds, loads, and gives the release library's weights bit for bit.
"""

import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from test_gpu_parity import assert_same, distorted, rect

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def rg():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import regridding_gb300

    return regridding_gb300


def test_undersized_chunk_slots_take_the_recovery_path(rg, monkeypatch):
    from regridding_gb300 import _device, workloads

    gi = distorted(257, 0.25, 0.02)
    go = workloads.perturb(rect(193, -1.05, 1.05))
    ref = rg.build_conservative_2d(gi, go).export_numpy()
    monkeypatch.setenv("RG_FAULT_CHUNK_SLOTS", "4")
    got = rg.build_conservative_2d(gi, go).export_numpy()
    for g, r, e in zip(got, ref, oracle.weights_conservative_2d(gi, go)):
        assert_same(g, r)
        assert_same(g, e)
    # batched builds take the same path for the whole batch
    rng = np.random.default_rng(12)
    pairs = [workloads.grid_pair(rng, side) for side in (40, 97, 150)]
    batched = _device.build_conservative_2d_batch(pairs)
    for (pgi, pgo), dw in zip(pairs, batched):
        for g, e in zip(dw.export_numpy(), oracle.weights_conservative_2d(pgi, pgo)):
            assert_same(g, e)


def test_debug_library_builds_and_matches():
    code = f"""
import sys
sys.path.insert(0, {ROOT!r})
sys.path.insert(0, {os.path.join(ROOT, 'tests')!r})
import numpy as np
import oracle
import regridding_gb300 as rg
from regridding_gb300 import _lib, workloads
assert _lib.library_path().endswith('_build_debug/libregrid_gb300.so'), _lib.library_path()
gi = workloads.distorted_grid(129, 0.3, 0.02)
go = workloads.perturb(workloads.rect_grid(97, -1.05, 1.05))
got = rg.build_conservative_2d(gi, go).export_numpy()
for g, e in zip(got, oracle.weights_conservative_2d(gi, go)):
    assert np.array_equal(g, e)
print('debug ok', _lib.load()._name)
"""
    env = dict(os.environ, RG_DEBUG="1")
    res = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "debug ok" in res.stdout
