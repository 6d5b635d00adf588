"""Minimal stand-in for ``numba`` so the reference meshoid source can be
imported as plain Python when generating golden vectors (numba is not
installed).  Decorators return the undecorated function, ``prange`` is
``range`` and ``vectorize`` wraps with ``np.vectorize``.  Test scaffolding
only: used by tests/golden/make_golden.py and nothing else.
"""
import numpy as np


def _passthrough(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    return lambda f: f


njit = jit = _passthrough


def vectorize(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return np.vectorize(args[0])
    return lambda f: np.vectorize(f)


def guvectorize(*args, **kwargs):
    return lambda f: f


prange = range


def get_num_threads():
    return 1


class _Signature:
    def __init__(self, name):
        self.name = name

    def __call__(self, *args):
        return (self.name, args)


float32 = _Signature("float32")
float64 = _Signature("float64")
