"""Import the upstream ``regridding`` package in its JIT-disabled (pure Python) mode.

Used only by ``make_golden.py`` in this directory to produce the committed
fixtures.  The upstream source tree is read in place; nothing is copied.
Its location is the environment variable ``REGRIDDING_REFERENCE`` (the
directory that holds the ``regridding`` package), e.g.

    REGRIDDING_REFERENCE=/path/to/regridding python tests/golden/make_golden.py
"""

import os
import sys

_SHIM = os.path.join(os.path.dirname(os.path.abspath(__file__)), "refshim")


def reference_root() -> str:
    root = os.environ.get("REGRIDDING_REFERENCE")
    if not root or not os.path.isdir(os.path.join(root, "regridding")):
        raise RuntimeError("set REGRIDDING_REFERENCE to the upstream source tree (the directory holding the "
                           "`regridding` package) to regenerate the fixtures")
    return root


def import_reference():
    REFERENCE_ROOT = reference_root()
    sys.dont_write_bytecode = True
    os.environ["NUMBA_DISABLE_JIT"] = "1"
    if _SHIM not in sys.path:
        sys.path.insert(0, _SHIM)
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    import regridding  # noqa: E402

    return regridding
