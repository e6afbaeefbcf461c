"""Macroscopic strain of the applied stress, E_bar_sigma = S sigma (cupymag/utils/sigma_matrices.py:25-46).

S is the cubic compliance with s11, s12, s44 (parameters.py:197-199).
"""
import numpy as np


def get_Ebar_sigma(params):
    S = np.zeros((6, 6))
    S[0, 0] = S[1, 1] = S[2, 2] = params.s11
    S[3, 3] = S[4, 4] = S[5, 5] = params.s44
    S[0, 1] = S[0, 2] = S[1, 0] = S[1, 2] = S[2, 0] = S[2, 1] = params.s12
    return S @ np.asarray(params.sigma, dtype=np.float64)
