"""cupyx.scipy.sparse stand-in: SciPy sparse (golden-vector generation only)."""
from scipy.sparse import coo_matrix, csr_matrix, identity, kron  # noqa: F401
