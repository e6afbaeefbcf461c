"""cupyx cg stand-in: the oracle's restatement of CuPy's cg (golden generation only)."""
import numpy as _np

CG_LOG = []


def cg(A, b, x0=None, tol=1e-5, maxiter=None, M=None, callback=None, atol=None):
    from oracle.cg import cg as _cg
    rec = []
    x, info = _cg(A, _np.asarray(b), x0=None if x0 is None else _np.asarray(x0), tol=tol, maxiter=maxiter,
                  record=rec)
    CG_LOG.append(rec[0])
    import cupy
    return cupy._wrap(x), info
