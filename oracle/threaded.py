"""Row-blocked CSR products on a thread pool, for timing the oracle on every host core.

TEST AND BASELINE INFRASTRUCTURE: used only by bench.py's CPU legs (`cpu_baseline`
and `--impl reference`), which time the oracle's restatement of the reference's
step (cupymag/core/Micromagnetics.py:110-307) at full size.  The reference's own
CPU arithmetic is CuPy swapped for NumPy/SciPy, and SciPy's CSR product is
single-threaded; it releases the GIL, so row blocks of one product run in
parallel on a thread pool.  Each row's sum is computed by the same routine in
the same order as in the undivided product, so results are bit-identical to
`A @ x`.
"""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import scipy.sparse as sp


class ThreadedCSR:
    """`A @ x` for a SciPy CSR matrix A, computed as `threads` row blocks on a shared pool."""

    def __init__(self, A, pool: ThreadPoolExecutor, threads: int):
        self.A = A.tocsr()
        self.shape = self.A.shape
        self.dtype = self.A.dtype
        self.pool = pool
        bounds = np.linspace(0, self.shape[0], max(1, threads) + 1).astype(np.int64)
        self.blocks = [(int(a), int(b), self._rows(int(a), int(b))) for a, b in zip(bounds[:-1], bounds[1:])
                       if b > a]

    def _rows(self, a, b):
        """Rows a..b-1 as a CSR matrix on views of A's data and indices (no copy of the non-zeros;
        the constructor copies, so the arrays are set on an empty matrix of the block's shape)."""
        ip = self.A.indptr
        s, e = int(ip[a]), int(ip[b])
        rows = sp.csr_matrix((b - a, self.shape[1]), dtype=self.dtype)
        rows.data = self.A.data[s:e]
        rows.indices = self.A.indices[s:e]
        rows.indptr = (ip[a:b + 1] - ip[a]).astype(self.A.indices.dtype)
        return rows

    def __matmul__(self, x):
        x = np.asarray(x)
        out = np.empty((self.shape[0],) + x.shape[1:], dtype=np.result_type(self.dtype, x.dtype))

        def run(block):
            a, b, rows = block
            out[a:b] = rows @ x

        list(self.pool.map(run, self.blocks))
        return out

    def dot(self, x):
        return self @ x


class ThreadedAxpy:
    """x + a * y in row blocks on a pool: element by element the same multiply and add as NumPy's
    `x + a * y` (and `x - a * y` as a = -a), so the result is bit-identical."""

    def __init__(self, pool: ThreadPoolExecutor, threads: int):
        self.pool = pool
        self.threads = max(1, threads)

    def __call__(self, x, a, y):
        n = x.shape[0]
        out = np.empty_like(x)
        bounds = np.linspace(0, n, self.threads + 1).astype(np.int64)

        def run(k):
            lo, hi = int(bounds[k]), int(bounds[k + 1])
            np.multiply(y[lo:hi], a, out=out[lo:hi])
            np.add(x[lo:hi], out[lo:hi], out=out[lo:hi])

        list(self.pool.map(run, range(self.threads)))
        return out


def host_threads() -> int:
    """Host cores this process may run on."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def threaded_operators(ops: dict, threads: int | None = None):
    """The operator dict with every sparse matrix wrapped in ThreadedCSR; returns (ops, pool, threads)."""
    threads = threads or host_threads()
    pool = ThreadPoolExecutor(max_workers=threads)
    out = {k: (ThreadedCSR(v, pool, threads) if sp.issparse(v) else v) for k, v in ops.items()}
    return out, pool, threads
