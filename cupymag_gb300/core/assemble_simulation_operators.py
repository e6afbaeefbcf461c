"""Mesh + operators for one run (drop-in for cupymag/core/assemble_simulation_operators.py:27-118).

``SimulationOperators(params)`` builds the mesh (FEMMesh of
cupymag/mesh/setup_FEM_mesh.py:42-95), the periodic DOF map and the defect
DOFs, and returns device CSR operators with the reference's method names:

* csr_demag_and_deriv() -> A_demag (DOF-0 anchored Laplacian), Fx, Fy, Fz, Deriv
* csr_GS()              -> A1 = alpha1 K + M, A2 = alpha2 K + M, F1 = M, with
                           defect rows/columns enforced (:67-85)
* csr_elasticity()      -> A_el (3 anchors), F_el, or (None, None) without ME
* volume_average()      -> VolumeAverage

Unlike the reference the parameters are an explicit object, not import-time
globals, so one process can hold several meshes (serving).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

from ..mesh.grids import HexGrid, TetraGrid, extract_defect_dofs
from ..physics import assembly as AS
from ..physics import structured_hex as SH
from ..utils.compute_derivatives import ComputeDerivatives
from ..utils.defect_shapes import get_defect_shape_function
from ..utils.device_csr import DeviceCSR
from ..utils.rot_111_matrices import get_M_matrix
from ..utils.volume_average import VolumeAverage


def _device_csr(indptr, indices, data, shape):
    nnz = data.numel()
    ip = indptr.to(torch.int64 if nnz >= 2 ** 31 else torch.int32)
    return DeviceCSR(ip.contiguous(), indices.contiguous(), data.contiguous(), shape)


DEVICE_COO_ELEMENTS = 200_000  # unstructured meshes at least this large assemble on the device


class SimulationOperators:
    def __init__(self, params, device=None, assembly="auto", mesh=None):
        self.p = params
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if mesh is not None:
            self.fem_grid = mesh
        elif params.grid_type == "Hex":
            self.fem_grid = HexGrid(params.Nx, params.Ny, params.Nz, params.Ndx, params.Ndy, params.Ndz,
                                    params.defect_center)
        elif params.grid_type == "Tet":
            params_shape = params.defect_parameters
            if params.defect_shape == "RotatedEllipsoid":
                params_shape = (params.defect_parameters, params.defect_rotation)
            fn = get_defect_shape_function(params.defect_shape, params_shape)
            self.fem_grid = TetraGrid(params.mesh_file, fn, params.defect_center)
        else:
            raise NotImplementedError(f"Grid type '{params.grid_type}' is not supported.")
        self.node_coords_np, self.elements_np = self.fem_grid.std_fem_mesh()
        self.global_id_np = self.fem_grid.build_periodic_node_map(self.node_coords_np)
        self.n_dof = int(self.global_id_np.max()) + 1
        self.n_nodes = self.node_coords_np.shape[0]
        self.n_elements = self.elements_np.shape[0]
        self.DefDOF = extract_defect_dofs(self.elements_np, self.global_id_np)
        self.alpha1 = params.alpha1
        self.alpha2 = params.alpha2
        g = self.fem_grid
        structured = isinstance(g, HexGrid) and min(g.Nx, g.Ny, g.Nz) >= 3
        if assembly in ("coo", "device"):
            structured = False
        elif assembly == "structured" and not structured:
            raise ValueError("structured assembly needs a hex grid with at least 3 cells per axis")
        self.structured = structured
        # unstructured meshes: host COO (SciPy) for small meshes, device COO for large ones
        self.device_coo = assembly == "device" or (assembly == "auto" and not structured
                                                    and self.n_elements >= DEVICE_COO_ELEMENTS)
        self._coo_ops = None
        self._elem = None

    # ------------------------------------------------------------------ helpers
    def _C(self):
        p = self.p
        return AS.stiffness_voigt(p.c11, p.c12, p.c44, get_M_matrix() if p.rot111 else None)

    def _coo(self):
        """Operators of the general COO path: SciPy CSR (host) or DeviceCSR (device assembly)."""
        if self._coo_ops is None:
            args = (self.node_coords_np, self.elements_np, self.global_id_np, self.n_dof, self.DefDOF, self.alpha1,
                    self.alpha2)
            kw = dict(ME=self.p.ME, C=self._C() if self.p.ME else None)
            if self.device_coo:
                from ..physics.device_assembly import assemble_device
                n = self.n_dof
                shapes = {"A_el": (3 * n, 3 * n), "F_el": (3 * n, 6 * n)}
                dev_ops = assemble_device(*args, device=self.device, **kw)
                self._coo_ops = {k: _device_csr(*v, shapes.get(k, (n, n))) for k, v in dev_ops.items()}
            else:
                self._coo_ops = AS.assemble_coo(*args, **kw)
        return self._coo_ops

    def _coo_op(self, name):
        A = self._coo()[name]
        return A if isinstance(A, DeviceCSR) else DeviceCSR.from_scipy(A, self.device)

    def _cell(self):
        """Element matrices of the unit cell at the origin (all cells are identical)."""
        if self._elem is None:
            el0 = self.elements_np[:1, :8]
            xe = self.node_coords_np[el0]
            K, M, F = AS.scalar_element_matrices(xe)
            self._elem = {"K": K[0], "M": M[0], "F": [f[0] for f in F]}
            if self.p.ME:
                Kel, Fel = AS.elastic_element_matrices(xe, self._C())
                self._elem["Kel"], self._elem["Fel"] = Kel[0], Fel[0]
        return self._elem

    def _scalar(self, Ke, anchors=(), defect=None, rows_only=False):
        g = self.fem_grid
        S = SH.stencil_from_element(Ke)[0, 0]
        ip, ix, dv = SH.scalar_csr(g.Nx, g.Ny, g.Nz, S, self.device)
        if anchors:
            ip, ix, dv = SH.anchor(ip, ix, dv, anchors)
        if defect is not None and len(defect):
            ip, ix, dv = SH.drop_defect(ip, ix, dv, defect, cols_too=not rows_only, unit_diag=not rows_only)
        return _device_csr(ip, ix, dv, (self.n_dof, self.n_dof))

    # ------------------------------------------------------------------ reference API
    def csr_demag_and_deriv(self):
        if self.structured:
            A = self._scalar(self._cell()["K"], anchors=(0,))
        else:
            A = self._coo_op("A_demag")
        return (A, *self.derivative_operators())

    def derivative_operators(self):
        """Fx, Fy, Fz and ComputeDerivatives over them (without the demag matrix)."""
        if self.structured:
            Fs = [self._scalar(f) for f in self._cell()["F"]]
        else:
            Fs = [self._coo_op(k) for k in ("Fx", "Fy", "Fz")]
        # the three derivative matrices share one pattern: keep one index copy
        for f in Fs[1:]:
            if f.same_pattern(Fs[0]):
                f.indptr, f.indices, f._struct = Fs[0].indptr, Fs[0].indices, None
        return Fs[0], Fs[1], Fs[2], ComputeDerivatives(*Fs)

    def elastic_rhs_operator(self):
        """F_el alone (the stencil path solves A_el matrix-free); None without ME."""
        if not self.p.ME:
            return None
        if self.structured:
            g, e, n = self.fem_grid, self._cell(), self.n_dof
            SF = SH.stencil_from_element(e["Fel"], 3, 6)
            ip, ix, dv = SH.elastic_F_csr(g.Nx, g.Ny, g.Nz, SF, self.device)
            ip, ix, dv = SH.anchor(ip, ix, dv, (0, n, 2 * n), cols_too=False, diag_one=False)
            return _device_csr(ip, ix, dv, (3 * n, 6 * n))
        return self._coo_op("F_el")

    def csr_GS(self):
        if self.structured:
            e = self._cell()
            A1 = self._scalar(e["K"] * self.alpha1 + e["M"], defect=self.DefDOF)
            A2 = self._scalar(e["K"] * self.alpha2 + e["M"], defect=self.DefDOF)
            F1 = self._scalar(e["M"], defect=self.DefDOF, rows_only=True)
            return A1, A2, F1
        return tuple(self._coo_op(k) for k in ("A1", "A2", "F1"))

    def csr_elasticity(self):
        if not self.p.ME:
            return None, None
        n = self.n_dof
        if self.structured:
            g = self.fem_grid
            e = self._cell()
            SA = SH.stencil_from_element(e["Kel"], 3, 3)
            ip, ix, dv = SH.elastic_A_csr(g.Nx, g.Ny, g.Nz, SA, self.device)
            ip, ix, dv = SH.anchor(ip, ix, dv, (0, n, 2 * n))
            A_el = _device_csr(ip, ix, dv, (3 * n, 3 * n))
            return A_el, self.elastic_rhs_operator()
        return self._coo_op("A_el"), self._coo_op("F_el")

    def stencil_derivatives(self):
        """Matrix-free Fx, Fy, Fz (StencilDerivatives: Hd, demag right-hand side, strain) for structured hex grids."""
        from ..utils.stencil_derivatives import StencilDerivatives
        if not self.structured:
            raise ValueError("stencil derivatives need a structured hex grid (at least 3 cells per axis)")
        g, e = self.fem_grid, self._cell()
        fx, fy, fz = (SH.stencil_from_element(f).reshape(-1) for f in e["F"])
        return StencilDerivatives(g.Nx, g.Ny, g.Nz, fx, fy, fz, self.device)

    def stencil_coupling(self):
        """Matrix-free F_el (StencilCoupling, anchor rows of DOF 0 empty); None without ME."""
        from ..utils.stencil_derivatives import StencilCoupling
        if not self.p.ME:
            return None
        if not self.structured:
            raise ValueError("the stencil coupling needs a structured hex grid (at least 3 cells per axis)")
        g, e = self.fem_grid, self._cell()
        SF = SH.stencil_from_element(e["Fel"], 3, 6).reshape(3, 6, 27)
        return StencilCoupling(g.Nx, g.Ny, g.Nz, SF.reshape(-1), anchor=True, device=self.device)

    def stencil_operators(self):
        """Matrix-free forms of A_demag, A1, A2, F1 (and A_el with ME) for structured hex grids."""
        from ..utils.stencil_operator import COL_EXCLUDED, ROW_IDENTITY, ROW_ZERO, StencilOperator
        if not self.structured:
            raise ValueError("stencil operators need a structured hex grid (at least 3 cells per axis)")
        g, e, n = self.fem_grid, self._cell(), self.n_dof
        st = lambda K: SH.stencil_from_element(K).reshape(-1)  # noqa: E731
        mk = lambda coef, flags=None: StencilOperator(g.Nx, g.Ny, g.Nz, coef, flags, self.device)  # noqa: E731
        pin = StencilOperator.flags_for(n, [0], ROW_IDENTITY | COL_EXCLUDED)
        dfl = StencilOperator.flags_for(n, self.DefDOF, ROW_IDENTITY | COL_EXCLUDED) if len(self.DefDOF) else None
        frow = StencilOperator.flags_for(n, self.DefDOF, ROW_ZERO) if len(self.DefDOF) else None
        out = {"A_demag": mk(st(e["K"]), pin),
               "A1": mk(st(e["K"] * self.alpha1 + e["M"]), dfl),
               "A2": mk(st(e["K"] * self.alpha2 + e["M"]), dfl),
               "F1": mk(st(e["M"]), frow)}
        if self.p.ME:
            out["A_el"] = mk(SH.stencil_from_element(e["Kel"], 3, 3).reshape(-1), pin)
        return out

    def stencil_step_operators(self):
        """Every operator of an LLG step in matrix-free form, as the tuple LLGSolver(ops=...) takes:
        (A_demag, Fx, Fy, Fz, Deriv, A1, A2, F1, A_el, F_el, Avg) with Fx = Fy = Fz = None (the
        derivatives act through Deriv).  The objects are read-only during a step, so runs of identical
        grids and materials can share one tuple."""
        so = self.stencil_operators()
        return (so["A_demag"], None, None, None, self.stencil_derivatives(), so["A1"], so["A2"], so["F1"],
                so.get("A_el"), self.stencil_coupling(), self.volume_average())

    def volume_average(self):
        return VolumeAverage(self.node_coords_np, self.elements_np, self.global_id_np, device=self.device)

    # host copies (tests, CPU baseline)
    def host_operators(self):
        """All operators as SciPy CSR matrices on the host."""
        A, Fx, Fy, Fz, _ = self.csr_demag_and_deriv()
        A1, A2, F1 = self.csr_GS()
        out = {"A_demag": A, "Fx": Fx, "Fy": Fy, "Fz": Fz, "A1": A1, "A2": A2, "F1": F1}
        A_el, F_el = self.csr_elasticity()
        if A_el is not None:
            out.update(A_el=A_el, F_el=F_el)
        return {k: v.to_scipy() for k, v in out.items()}
