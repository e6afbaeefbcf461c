"""CPU oracle for the Gauss-Seidel-projection LLG step -- TEST INFRASTRUCTURE.

This package is a NumPy/SciPy restatement of the reference's algorithm for the
LLG time step (cupymag/core/Micromagnetics.py:110-307) and everything it
consumes: mesh and periodic DOF map, FEM assembly, the volume average, the
unpreconditioned CG of cupyx.scipy.sparse.linalg.cg, the eigenstrain and
strain operators.  Each function cites the reference file:line it follows.

It is only used as a checker: by tests/, by ``__graft_entry__.smoke()`` and
by the CPU-baseline leg of ``bench.py``.  The product package never imports
it, and the product has no CPU fallback.

Parity pinning: the restatement is checked against golden vectors generated
by running the reference's own Python sources (with test-only stand-ins for
cupy/numba/yaml/h5py/meshio/pandas), see tests/golden/make_golden.py.  The CG
itself lives in CuPy (third-party, absent here); its algorithm is restated
from CuPy's published cg (cupyx/scipy/sparse/linalg/_iterative.py, CuPy
v10-v13) and anchored on the reference's call sites
(cupymag/solvers/linear_solvers.py:59-74).
"""
