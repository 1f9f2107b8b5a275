class List(list):
    """A ``numba.typed.List`` in JIT-disabled mode behaves as a Python list."""
