"""Physical constants used by the nondimensionalisation.

Same values as the reference (cupymag/core/constants.py:17-30): vacuum
permeability in H/m and the gyromagnetic ratio in rad/(s*T), plus the square
roots used by the [111] rotation matrices.
"""
import math

MU0 = 1.25663706127e-6
GAMMA = 1.76e11

sqrt2 = math.sqrt(2.0)
sqrt3 = math.sqrt(3.0)
sqrt6 = math.sqrt(6.0)

inv_sqrt2 = 1.0 / sqrt2
inv_sqrt3 = 1.0 / sqrt3
inv_sqrt6 = 1.0 / sqrt6
