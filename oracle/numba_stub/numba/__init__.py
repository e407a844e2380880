"""Pass-through stand-in for ``numba`` (test infrastructure only).

numba need not be installed.  The reference package
decorates its kernels with ``@jit(nopython=True)``; numba without fast-math
compiles them to IEEE FP64 without FMA contraction, which is exactly what the
plain CPython interpreter computes.  This stub makes ``jit`` the identity so
the reference modules import and run interpreted, with the same numerics.
Only the golden-vector generator under ``tests/golden`` puts it on sys.path.
"""


def jit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]

    def wrap(fn):
        return fn

    return wrap


njit = jit
