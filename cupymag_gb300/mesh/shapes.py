"""Shape functions and quadrature of the trilinear hex and the linear tet.

Hex (cupymag/mesh/ShapeHex.py): corners in the order of ShapeHex.py:289-300,
2x2x2 Gauss rule at the point 0.57735026919 (ShapeHex.py:271-286, loop order
r, s, t).  Assembly uses the values of N and dN/dxi at those points rounded to
12 decimals (the tables of ShapeHex.py:302-393 are exactly that); the volume
average evaluates the formulas unrounded.
Tet (cupymag/mesh/ShapeTet.py): 4-point rule a = 0.58541020, b = 0.13819660,
weights 1/24; N at point g is a at node g and b elsewhere (ShapeTet.py:243-248);
dN/dxi constant.
"""
import numpy as np

HEX_CORNERS = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                        [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=np.float64)
HEX_OFFSETS = ((HEX_CORNERS + 1) // 2).astype(np.int64)  # corner offsets within the cell
_G = 0.57735026919


def hex_gauss_points():
    p = np.array([(a, b, c) for a in (-_G, _G) for b in (-_G, _G) for c in (-_G, _G)], dtype=np.float64)
    return p, np.ones(8)


def hex_N(r, s, t):
    c = HEX_CORNERS
    return (1 + c[:, 0] * r) * (1 + c[:, 1] * s) * (1 + c[:, 2] * t) / 8.0


def hex_dN(r, s, t):
    c = HEX_CORNERS
    return np.stack([c[:, 0] * (1 + c[:, 1] * s) * (1 + c[:, 2] * t) / 8.0,
                     c[:, 1] * (1 + c[:, 0] * r) * (1 + c[:, 2] * t) / 8.0,
                     c[:, 2] * (1 + c[:, 0] * r) * (1 + c[:, 1] * s) / 8.0], axis=1)


def hex_assembly_tables():
    pts, w = hex_gauss_points()
    dN = np.round(np.stack([hex_dN(*q) for q in pts]), 12)
    N = np.round(np.stack([hex_N(*q) for q in pts]), 12)
    return dN, N, w


TET_A, TET_B = 0.58541020, 0.13819660


def tet_gauss_points():
    a, b = TET_A, TET_B
    return np.array([[b, b, b], [a, b, b], [b, a, b], [b, b, a]]), np.full(4, 1.0 / 24.0)


def tet_N(r, s, t):
    return np.array([1.0 - r - s - t, r, s, t])


def tet_dN(r=0.0, s=0.0, t=0.0):
    return np.array([[-1.0, -1.0, -1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])


def tet_assembly_tables():
    N = np.full((4, 4), 0.1381966)
    np.fill_diagonal(N, 0.5854102)
    return np.broadcast_to(tet_dN(), (4, 4, 3)).copy(), N, tet_gauss_points()[1]
