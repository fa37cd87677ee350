"""Test-only stand-in for numba, used solely to import the reference solver in
a container where numba is not installed (golden-fixture generation).

`njit` returns the function unchanged, `prange` is `range`: the reference's
kernels then run as plain Python in the same float64 arithmetic and the same
loop order.
"""

prange = range


class _Config:
    NUMBA_NUM_THREADS = 1


config = _Config()


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(fn):
        return fn

    return wrap


jit = njit


def set_num_threads(n):
    return None


def get_num_threads():
    return 1
