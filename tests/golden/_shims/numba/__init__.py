"""numba stand-in: decorators are identity, types are subscriptable markers."""


class _Type:
    def __getitem__(self, item):
        return self

    def __call__(self, *a, **k):
        return self


float64 = _Type()
float32 = _Type()
int32 = _Type()
int64 = _Type()


def njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    return lambda f: f


jit = njit
