"""Unpreconditioned conjugate gradient with cupyx.scipy.sparse.linalg.cg semantics.

The reference solves every system through ``solve_cg``
(cupymag/solvers/linear_solvers.py:20-74), which calls CuPy's ``cg``
(third-party; ``cupy>=10.0.0`` in requirements.txt:3, not vendored and not
installed here).  CuPy's published algorithm, restated:

* x = 0 when x0 is None, else a copy of x0;
* if ||b|| == 0 return (b, 0) immediately;
* atol = tol * ||b||;  r = b - A x;
* loop while iters < maxiter: rho = r.r; p = r (first) or r + (rho/rho_old) p;
  q = A p; alpha = rho / (p.q); x += alpha p; r -= alpha q; iters += 1;
  stop when ||r|| <= atol  (checked after the update, so a converged warm
  start still does one iteration);
* info = iters if maxiter was reached without convergence, else 0.

``solve_cg`` passes x0 only when use_init is true and raises RuntimeError
with the residual ||b - A x|| when info != 0 (linear_solvers.py:59-74).
"""
import numpy as np


def _axpy(x, a, y):
    return x + a * y


def cg(A, b, x0=None, tol=1e-5, maxiter=None, record=None, axpy=None, dot=None):
    """axpy(x, a, y) -> x + a * y (element-wise; a threaded one must round the same way).

    dot(a, b) -> a.b for the two CG inner products (rho and p.q); the default is
    np.dot.  Tests pass another summation order to measure how far a
    trajectory moves when only the rounding of one reduction changes."""
    axpy = axpy or _axpy
    dot = dot or np.dot
    n = A.shape[0]
    if maxiter is None:
        maxiter = n * 10
    bnorm = np.linalg.norm(b)
    if bnorm == 0:
        if record is not None:
            record.append(0)
        return b.copy(), 0
    atol = tol * float(bnorm)
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    r = b - A @ x
    iters = 0
    rho = 0.0
    p = None
    resid = np.inf
    while iters < maxiter:
        rho1 = rho
        rho = dot(r, r)
        if iters == 0:
            p = r.copy()
        else:
            p = axpy(r, rho / rho1, p)
        q = A @ p
        alpha = rho / dot(p, q)
        x = axpy(x, alpha, p)
        r = axpy(r, -alpha, q)
        iters += 1
        resid = np.linalg.norm(r)
        if resid <= atol:
            break
    info = 0
    if iters == maxiter and not (resid <= atol):
        info = iters
    if record is not None:
        record.append(iters)
    return x, info


def solve_cg(A, b, M=None, x0=None, tol=1e-7, maxiter=5000, use_init=False, system=None, record=None, dot=None):
    x, info = cg(A, b, x0=(x0 if use_init else None), tol=tol, maxiter=maxiter, record=record, dot=dot)
    if info == 0:
        return x
    rnorm = np.linalg.norm(b - A @ x)
    if system is not None:
        msg = f"Error! CG for {system} did not converge. info={info}, residual={rnorm}."
    else:
        msg = f"Error! CG did not converge. info={info}, residual={rnorm}."
    raise RuntimeError(msg)
