"""Pure-Python stand-in for the few ``numba`` names the reference imports.

The reference library's own CI runs its whole test suite with
``NUMBA_DISABLE_JIT=1``, i.e. every ``@numba.njit`` function executes as plain
Python.  numba itself is not installed here, so this shim supplies exactly that
mode: ``njit`` is an identity decorator, ``prange`` is ``range``, typed lists
are Python lists.  It is only ever used to import the reference in order to
generate golden fixtures; nothing in the product imports it.
"""

from . import typed, types  # noqa: F401


def _decorator(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(func):
        return func

    return wrap


njit = _decorator
jit = _decorator
prange = range


def literal_unroll(x):
    return x
