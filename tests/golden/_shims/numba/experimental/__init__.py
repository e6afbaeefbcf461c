def jitclass(spec=None, *a, **k):
    if isinstance(spec, type):
        return spec
    return lambda cls: cls
