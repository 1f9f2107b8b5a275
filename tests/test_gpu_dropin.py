"""Drop-in behaviours of the public functions that the upstream's users rely
on beyond the numbers: writable weight arrays that can be edited in place
(and are then applied as edited), and the upstream's method names for 1D
find_indices (`regridding/_find_indices/_find_indices.py:112-125`)."""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rg():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import regridding_gb300

    return regridding_gb300


def test_weights_are_writable_and_edits_are_applied(rg):
    from regridding_gb300 import workloads

    gi, go, values = workloads.cfg1()
    w = rg.weights(gi, go, method="conservative")
    (ii, oo, vv), = w[0].reshape(-1)
    assert ii.flags.writeable and oo.flags.writeable and vv.flags.writeable
    first = rg.regrid_from_weights(*w, values_input=values)
    again = rg.regrid_from_weights(*w, values_input=values)  # device copy reused
    np.testing.assert_array_equal(first, again)
    vv *= 2.0  # in place, as a user of the upstream may
    doubled = rg.regrid_from_weights(*w, values_input=values)
    np.testing.assert_array_equal(doubled, oracle.apply(ii, oo, vv, values.reshape(8, -1), 48 * 48).reshape(8, 48, 48))
    np.testing.assert_allclose(doubled, 2 * first, rtol=1e-15)
    oo[:] = oo[::-1].copy()  # indices edited too
    moved = rg.regrid_from_weights(*w, values_input=values)
    np.testing.assert_array_equal(moved, oracle.apply(ii, oo, vv, values.reshape(8, -1), 48 * 48).reshape(8, 48, 48))


def test_read_only_weights_keep_their_device_copy(rg):
    from regridding_gb300 import _device, workloads

    gi, go, values = workloads.cfg1()
    w = rg.weights(gi, go, method="conservative")
    element = w[0].reshape(-1)[0]
    for a in element:
        a.flags.writeable = False
    rg.regrid_from_weights(*w, values_input=values)
    dw = _device.lookup(element, 64 * 64, 48 * 48)
    assert dw is not None
    rg.regrid_from_weights(*w, values_input=values)
    assert _device.lookup(element, 64 * 64, 48 * 48) is dw


def test_find_indices_1d_method_names(rg):
    x = np.linspace(0, 1, 11)
    p = np.array([0.05, 0.5, 2.0])
    for method in ("brute", "searchsorted"):
        (got,) = rg.find_indices((x,), (p,), method=method)
        assert got.tolist() == [0, 4, np.iinfo(int).max]
    for method in ("exhaustive", "secant", "bisect"):
        with pytest.raises(ValueError, match="not recognized"):
            rg.find_indices((x,), (p,), method=method)
