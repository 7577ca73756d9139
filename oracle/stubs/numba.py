"""Test-only stand-in for numba so the reference imports without it.

`njit` returns the function unchanged and `prange` is `range`: the reference
then runs as plain NumPy/Python.  Used only by the golden-vector generator.
"""


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def deco(f):
        return f

    return deco


jit = njit
prange = range
