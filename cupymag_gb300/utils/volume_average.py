"""Volume averages on the GPU (drop-in for cupymag/utils/volume_average.py:69-216).

The reference integrates per element, per Gauss point:
<f> = sum_e sum_g (sum_b N_gb f[cdof_eb]) |detJ_eg| w_g / sum_e sum_g |detJ_eg| w_g,
with detJ computed from corner coordinates gathered by DOF id,
``coords[global_id[elements]]`` (volume_average.py:76,108) -- a quirk kept
here because every <m>, <E> and hysteresis value depends on it.  That sum is
linear in f, so it is folded once at setup into one weight per DOF,
w_d = sum over (e,b) with cdof_eb = d of sum_g N_gb |detJ_eg| w_g, and the
step-time average is a single weighted reduction kernel, <f> = (w . f) / V.
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _native as N
from ..mesh import shapes


_BLOCK = 1 << 18  # elements per block of the weight computation


def dof_weights(coords, elements, gid, n, defect_flag=None):
    nen = elements.shape[1] - 1
    cdof = gid[elements[:, :nen]].astype(np.int64)
    if nen == 8:
        pts, w = shapes.hex_gauss_points()
        Nf, dNf = shapes.hex_N, shapes.hex_dN
    else:
        pts, w = shapes.tet_gauss_points()
        Nf, dNf = shapes.tet_N, shapes.tet_dN
    ng = len(pts)
    # dN of every Gauss point side by side: J for all points is one GEMM per block
    dN = np.concatenate([dNf(r, s, t)[:nen] for (r, s, t) in pts], axis=1)  # (nen, 3*ng), column 3g + j
    Nt = np.stack([Nf(r, s, t) for (r, s, t) in pts])                        # (ng, nen)
    Ne = len(cdof)
    contrib = np.empty((Ne, nen))
    vol_e = np.empty(Ne)
    for e0 in range(0, Ne, _BLOCK):
        cc = coords[cdof[e0:e0 + _BLOCK]]                                    # (B, nen, 3)
        B = len(cc)
        J = (cc.transpose(0, 2, 1).reshape(B * 3, nen) @ dN).reshape(B, 3, ng, 3)  # J[e, k, g, j]
        a = lambda k, j: J[:, k, :, j]  # noqa: E731
        # cofactor expansion along the first row, as volume_average.py:123-125
        det = (a(0, 0) * (a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1))
               - a(0, 1) * (a(1, 0) * a(2, 2) - a(1, 2) * a(2, 0))
               + a(0, 2) * (a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0)))
        vw = np.abs(det) * w[None, :]
        contrib[e0:e0 + B] = vw @ Nt
        vol_e[e0:e0 + B] = vw.sum(axis=1)
    if defect_flag is not None:
        keep = 1.0 - np.asarray(defect_flag, dtype=np.float64)
        contrib *= keep[:, None]
        vol_e = vol_e * keep
    wd = np.bincount(cdof.ravel(), weights=contrib.ravel(), minlength=n)
    return wd, float(np.sum(vol_e))


class VolumeAverage:
    def __init__(self, coords, elements, global_id, device=None):
        self.coords = np.asarray(coords)
        self.elements = np.asarray(elements)
        self.global_id = np.asarray(global_id)
        self.n = int(self.global_id.max()) + 1
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        w, V = dof_weights(self.coords, self.elements, self.global_id, self.n)
        self._set = {None: self._upload(w, V)}
        self.scratch = torch.zeros(N.lib().cpm_volavg_scratch_doubles(6), dtype=torch.float64, device=self.device)

    def _upload(self, w, V):
        if abs(V) < 1e-6:
            print("WARNING: Total volume is very small, results may be unstable")
            V = max(abs(V), 1e-6)
        return torch.as_tensor(w, dtype=torch.float64, device=self.device), float(V)

    def weights(self, defect_flag=None):
        key = None if defect_flag is None else "nodefect"
        if key not in self._set:
            w, V = dof_weights(self.coords, self.elements, self.global_id, self.n, defect_flag=self.elements[:, -1])
            self._set[key] = self._upload(w, V)
        return self._set[key]

    def average_into(self, f, out, R9=None, defect_flag=None):
        w, V = self.weights(defect_flag)
        nc = 1 if f.dim() == 1 else f.shape[1]
        N.check(N.lib().cpm_volavg(self.n, nc, f.data_ptr(), w.data_ptr(), V,
                                   None if R9 is None else R9.data_ptr(), out.data_ptr(), self.scratch.data_ptr(),
                                   N.stream_ptr()), "cpm_volavg")
        return out

    def compute_average_field_gpu(self, m, defect_flag=None):
        """<m> over the mesh: scalar -> 0-d tensor, (n,c) -> (c,) tensor (volume_average.py:155-216)."""
        m = torch.as_tensor(m, dtype=torch.float64, device=self.device).contiguous()
        nc = 1 if m.dim() == 1 else m.shape[1]
        if nc not in (1, 3, 6):
            return torch.stack([self.compute_average_field_gpu(m[:, c].contiguous(), defect_flag) for c in range(nc)])
        out = torch.empty(nc, dtype=torch.float64, device=self.device)
        self.average_into(m, out, defect_flag=defect_flag)
        return out[0] if m.dim() == 1 else out
