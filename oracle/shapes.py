"""Shape-function tables of the trilinear hex and linear tet (oracle).

Hex (cupymag/mesh/ShapeHex.py):
* Gauss points: 2x2x2 rule with the point written as 0.57735026919 (not the
  exact 1/sqrt(3)), loop order r outer, s, t inner (ShapeHex.py:271-286);
* assembly uses tables of N and dN/dxi at those points rounded to 12 decimals
  (ShapeHex.py:302-393);
* the volume average evaluates the formulas at the points, unrounded
  (ShapeHex.py:25-146, used by volume_average.py:96-153).
Tet (cupymag/mesh/ShapeTet.py):
* 4-point rule a=0.58541020, b=0.13819660, w=1/24 (ShapeTet.py:204-229);
* N table is the permutation (a, b, b, b) per point, dN constant
  (ShapeTet.py:243-255).
"""
import numpy as np

HEX_CORNERS = np.array([
    [-1, -1, -1], [+1, -1, -1], [+1, +1, -1], [-1, +1, -1],
    [-1, -1, +1], [+1, -1, +1], [+1, +1, +1], [-1, +1, +1]], dtype=np.float64)

HEX_GP_1D = 0.57735026919


def hex_gauss():
    pts = []
    for rx in (-HEX_GP_1D, HEX_GP_1D):
        for ry in (-HEX_GP_1D, HEX_GP_1D):
            for rz in (-HEX_GP_1D, HEX_GP_1D):
                pts.append((rx, ry, rz))
    return np.array(pts, dtype=np.float64), np.ones(8, dtype=np.float64)


def hex_N(r, s, t):
    c = HEX_CORNERS
    return (1 + c[:, 0] * r) * (1 + c[:, 1] * s) * (1 + c[:, 2] * t) / 8.0


def hex_dN(r, s, t):
    c = HEX_CORNERS
    d = np.empty((8, 3))
    d[:, 0] = c[:, 0] * (1 + c[:, 1] * s) * (1 + c[:, 2] * t) / 8.0
    d[:, 1] = c[:, 1] * (1 + c[:, 0] * r) * (1 + c[:, 2] * t) / 8.0
    d[:, 2] = c[:, 2] * (1 + c[:, 0] * r) * (1 + c[:, 1] * s) / 8.0
    return d


def hex_tables():
    """(dN_table (8,8,3), N_table (8,8)) rounded to 12 decimals."""
    pts, _ = hex_gauss()
    dN = np.stack([hex_dN(*p) for p in pts])
    N = np.stack([hex_N(*p) for p in pts])
    return np.round(dN, 12), np.round(N, 12)


TET_A = 0.58541020
TET_B = 0.13819660


def tet_gauss():
    a, b = TET_A, TET_B
    pts = np.array([[b, b, b], [a, b, b], [b, a, b], [b, b, a]], dtype=np.float64)
    return pts, np.ones(4, dtype=np.float64) / 24.0


def tet_N(r, s, t):
    return np.array([1.0 - r - s - t, r, s, t])


def tet_dN(r=0.0, s=0.0, t=0.0):
    return np.array([[-1.0, -1.0, -1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])


def tet_tables():
    N = np.full((4, 4), 0.1381966)
    np.fill_diagonal(N, 0.5854102)
    dN = np.stack([tet_dN() for _ in range(4)])
    return dN, N
