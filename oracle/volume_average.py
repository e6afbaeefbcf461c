"""Volume average (oracle restatement of cupymag/utils/volume_average.py:69-216).

Keeps the reference's behaviour exactly, including that the corner
coordinates used for detJ are gathered by DOF id, ``coords[global_id[elem]]``
(volume_average.py:76,108), and that detJ is taken in absolute value
(volume_average.py:127).  N and dN are the unrounded formulas at the Gauss
points (volume_average.py:96-153).
"""
import numpy as np

from . import shapes


class VolumeAverage:
    def __init__(self, coords, elements, gid):
        nen = elements.shape[1] - 1
        self.nen = nen
        self.corner_dofs = gid[elements[:, :nen]]
        self.defect_flags = elements[:, -1]
        if nen == 8:
            pts, w = shapes.hex_gauss()
            Nf, dNf = shapes.hex_N, shapes.hex_dN
        else:
            pts, w = shapes.tet_gauss()
            Nf, dNf = shapes.tet_N, shapes.tet_dN
        self.W = w
        cc = coords[self.corner_dofs]  # quirk: coordinates gathered by DOF id
        self.detJ = np.zeros((elements.shape[0], len(w)))
        for g, (r, s, t) in enumerate(pts):
            dN = dNf(r, s, t)[:nen]
            J = np.einsum("enk,nj->ekj", cc, dN)
            # cofactor expansion along the first row (volume_average.py:123-125)
            det = (J[:, 0, 0] * (J[:, 1, 1] * J[:, 2, 2] - J[:, 1, 2] * J[:, 2, 1])
                   - J[:, 0, 1] * (J[:, 1, 0] * J[:, 2, 2] - J[:, 1, 2] * J[:, 2, 0])
                   + J[:, 0, 2] * (J[:, 1, 0] * J[:, 2, 1] - J[:, 1, 1] * J[:, 2, 0]))
            self.detJ[:, g] = np.abs(det)
        self.N = np.stack([Nf(*p) for p in pts])  # (ngp, nen)

    def average(self, m, defect_flag=None):
        scalar = m.ndim == 1
        if scalar:
            m = m.reshape(-1, 1)
        cu = m[self.corner_dofs]  # (e, b, k)
        mgp = np.einsum("ebk,gb->egk", cu, self.N)
        vw = self.detJ * self.W
        pe = np.sum(mgp * vw[:, :, None], axis=1)
        pv = np.sum(vw, axis=1)
        if defect_flag is not None:
            keep = 1.0 - defect_flag.astype(np.float64)
            pe = pe * keep[:, None]
            vol = np.sum(pv * keep)
        else:
            vol = np.sum(pv)
        tot = np.sum(pe, axis=0)
        if abs(vol) < 1e-6:
            vol = max(abs(vol), 1e-6)
        avg = tot / vol
        return avg[0] if scalar else avg

    def dof_weights(self, n, defect_flag=None):
        """Per-DOF weights w and volume V with avg(f) = (w . f) / V."""
        vw = self.detJ * self.W
        keep = np.ones(len(vw)) if defect_flag is None else 1.0 - defect_flag.astype(np.float64)
        contrib = np.einsum("eg,gb->eb", vw, self.N) * keep[:, None]
        w = np.zeros(n)
        np.add.at(w, self.corner_dofs.ravel(), contrib.ravel())
        return w, float(np.sum(vw.sum(axis=1) * keep))
