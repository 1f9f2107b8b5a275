"""Import the upstream ``regridding`` package in its JIT-disabled (pure Python) mode.

Used only by ``make_golden.py`` in this directory to produce the committed
fixtures.  The upstream source tree is read in place; nothing is copied.
"""

import os
import sys

REFERENCE_ROOT = os.environ.get("REGRIDDING_REFERENCE", "/root/reference")
_SHIM = os.path.join(os.path.dirname(os.path.abspath(__file__)), "refshim")


def import_reference():
    sys.dont_write_bytecode = True
    os.environ["NUMBA_DISABLE_JIT"] = "1"
    if _SHIM not in sys.path:
        sys.path.insert(0, _SHIM)
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    import regridding  # noqa: E402

    return regridding
