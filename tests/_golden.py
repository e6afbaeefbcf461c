"""Helpers to load the golden fixtures written by tests/golden/make_golden.py."""
import json
import os

import numpy as np
import scipy.sparse as sp

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["hex_plain", "hex_me_rot", "hex_me_norot", "tet_me_rot"]
DRIVER = "hex_driver"


def load(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz"), allow_pickle=False))


def config(g):
    return json.loads(str(g["config_json"]))


def matrix(g, name):
    key = f"mat_{name}_data"
    if key not in g:
        return None
    return sp.csr_matrix((g[key], g[f"mat_{name}_indices"], g[f"mat_{name}_indptr"]),
                         shape=tuple(g[f"mat_{name}_shape"]))


def matrices(g):
    out = {}
    for nm in ["A_demag", "Fx", "Fy", "Fz", "A1", "A2", "F1", "A_el", "F_el"]:
        A = matrix(g, nm)
        if A is not None:
            out[nm] = A
    return out


def params(g):
    from cupymag_gb300.core.parameters import params_from_config
    return params_from_config(config(g))
