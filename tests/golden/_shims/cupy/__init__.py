"""cupy stand-in backed by NumPy (golden-vector generation only)."""
import numpy as _np


class ndarray(_np.ndarray):
    def get(self):
        return _np.asarray(self).copy()


def _wrap(x):
    if isinstance(x, _np.ndarray) and not isinstance(x, ndarray):
        return x.view(ndarray)
    if isinstance(x, tuple):
        return tuple(_wrap(v) for v in x)
    if isinstance(x, list):
        return [_wrap(v) for v in x]
    return x


class _Forward:
    def __init__(self, mod):
        self._mod = mod

    def __getattr__(self, name):
        obj = getattr(self._mod, name)
        if callable(obj) and not isinstance(obj, type):
            def f(*a, **k):
                return _wrap(obj(*a, **k))
            return f
        return obj


linalg = _Forward(_np.linalg)
random = _Forward(_np.random)


class _Cuda:
    @staticmethod
    def is_available():
        return True


cuda = _Cuda()


def asnumpy(x):
    return _np.asarray(x)


def get_array_module(*args):
    import sys
    return sys.modules[__name__]


def __getattr__(name):
    obj = getattr(_np, name)
    if callable(obj) and not isinstance(obj, type):
        def f(*a, **k):
            return _wrap(obj(*a, **k))
        return f
    return obj


float64 = _np.float64
float32 = _np.float32
int32 = _np.int32
int64 = _np.int64
