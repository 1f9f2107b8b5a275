"""``numba.types.int64(x)`` is a compile-time cast in numba; here it is ``int``."""

int64 = int
