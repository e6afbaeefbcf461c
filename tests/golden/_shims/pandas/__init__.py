"""pandas stand-in: the read_csv subset used by the reference's .nas reader."""
import numpy as np


class _Frame:
    def __init__(self, cols, data):
        self.cols = list(cols)
        self.data = data

    def __getitem__(self, key):
        if isinstance(key, list):
            return _Frame(key, {k: self.data[k] for k in key})
        return _Frame([key], {key: self.data[key]})

    def astype(self, t):
        return _Frame(self.cols, {k: np.asarray(self.data[k]).astype(t) for k in self.cols})

    def to_numpy(self, copy=False):
        if len(self.cols) == 1:
            return np.asarray(self.data[self.cols[0]])
        return np.stack([np.asarray(self.data[k]) for k in self.cols], axis=1)


def read_csv(buf, names=None, sep=",", skipinitialspace=False, dtype=None, header=None, engine=None):
    rows = [ln.split(sep) for ln in buf.getvalue().splitlines() if ln.strip()]
    if skipinitialspace:
        rows = [[c.strip() for c in r] for r in rows]
    data = {nm: [r[i] if i < len(r) else "" for r in rows] for i, nm in enumerate(names)}
    return _Frame(names, data)
