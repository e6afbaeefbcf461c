"""Simulation parameters: config schema -> nondimensional scalars.

Restates cupymag/core/parameters.py:59-224 as an explicit object instead of
module-level globals loaded at import time.  One process can therefore hold
several runs with different configs (the serving loop needs that), and
importing this module has no side effects.

Nondimensionalisation (parameters.py:179-224):

* psi0 = MU0 * Ms^2; K1, A, c_ij and the applied stresses are divided by psi0;
* compliance s11, s12, s44 of the cubic crystal (parameters.py:197-199);
* magnetoelastic constants elasC1..3 (parameters.py:202-205);
* dt = timestep * MU0 * GAMMA * Ms / (1 + alpha^2);
* astar = 2 A / ld^2, alpha (exchange) = astar * dt;
* applied fields are divided by Ms.
"""
from __future__ import annotations

import math
import os
import sys
from dataclasses import dataclass, field, replace
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

from .config_loader import ConfigLoader
from .constants import GAMMA, MU0


def _validate_parameters(ms, ld, timestep, AA_raw, alpha_damp):
    """Positivity checks of parameters.py:26-36 (same messages)."""
    if ms <= 0:
        raise ValueError("Saturation magnetization must be positive")
    if ld <= 0:
        raise ValueError("Characteristic length must be positive")
    if timestep <= 0:
        raise ValueError("Timestep must be positive")
    if AA_raw <= 0:
        raise ValueError("Exchange constant must be positive")
    if alpha_damp < 0:
        raise ValueError("Damping constant alpha must be non-negative")


def _safe_divide(numerator, denominator, operation_name):
    """Guarded division of parameters.py:39-42."""
    if abs(denominator) < 1e-30:
        raise ValueError(f"Division by zero in {operation_name}: {denominator}")
    return numerator / denominator


@dataclass
class SimParams:
    """All scalars one LLG run needs, raw (SI) and nondimensional."""

    # raw physics
    ms: float = 1.2e6
    AA_raw: float = 1.5e-11
    K1_raw: float = 2.0e4
    c11_raw: float = 0.0
    c12_raw: float = 0.0
    c44_raw: float = 0.0
    lambda100: float = 0.0
    lambda111: float = 0.0
    N_x: float = 1.0 / 3.0
    N_y: float = 1.0 / 3.0
    N_z: float = 1.0 / 3.0
    Hext_raw: Sequence[float] = (0.0, 0.0, 0.0)
    dHext_raw: Sequence[float] = (0.0, 0.0, 0.0)
    sigma_raw: Sequence[float] = (0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    rot111: bool = False
    ME: bool = False
    ld: float = 10.0e-9
    # grid
    grid_type: str = "Hex"
    Nx: int = 0
    Ny: int = 0
    Nz: int = 0
    Ndx: int = 0
    Ndy: int = 0
    Ndz: int = 0
    defect_center: Optional[Sequence[float]] = None
    mesh_file: Optional[str] = None
    defect_shape: Optional[str] = None
    defect_parameters: Optional[Sequence[float]] = None
    defect_rotation: Optional[Sequence[Sequence[float]]] = None
    # simulation
    precision: str = "DP"
    timestep: float = 1e-12
    alpha_damp: float = 0.1
    LLG_accuracy_factor: float = 5e-10
    tol: float = 1e-10
    maxiter: int = 5000
    use_init_factor: float = 100.0
    restart: bool = False
    restart_m: Optional[str] = None
    initial_magnetization: Optional[Sequence[float]] = (1.0, 0.0, 0.0)
    stop_direction: Sequence[float] = (1.0, 0.0, 0.0)
    stop_value: float = -0.95
    # output
    output_dir: str = "."
    write_m: bool = True
    save_frequency: int = 1000
    vtu_alpha: float = 0.05
    config_path: Optional[str] = None

    # derived (filled by finalize())
    psi0: float = field(default=0.0, init=False)
    K1: float = field(default=0.0, init=False)
    AA: float = field(default=0.0, init=False)
    c11: float = field(default=0.0, init=False)
    c12: float = field(default=0.0, init=False)
    c44: float = field(default=0.0, init=False)
    sigma: tuple = field(default=(0.0,) * 6, init=False)
    s11: float = field(default=0.0, init=False)
    s12: float = field(default=0.0, init=False)
    s44: float = field(default=0.0, init=False)
    elasC1: float = field(default=0.0, init=False)
    elasC2: float = field(default=0.0, init=False)
    elasC3: float = field(default=0.0, init=False)
    dt: float = field(default=0.0, init=False)
    astar: float = field(default=0.0, init=False)
    alpha: float = field(default=0.0, init=False)
    Hext: tuple = field(default=(0.0, 0.0, 0.0), init=False)
    dHext: tuple = field(default=(0.0, 0.0, 0.0), init=False)

    def finalize(self) -> "SimParams":
        """Compute the nondimensional scalars (parameters.py:176-224)."""
        _validate_parameters(self.ms, self.ld, self.timestep, self.AA_raw, self.alpha_damp)
        psi0 = MU0 * self.ms ** 2
        self.psi0 = psi0
        self.K1 = _safe_divide(self.K1_raw, psi0, "K1 normalization")
        self.AA = _safe_divide(self.AA_raw, psi0, "AA normalization")
        self.c11 = _safe_divide(self.c11_raw, psi0, "c11 normalization")
        self.c12 = _safe_divide(self.c12_raw, psi0, "c12 normalization")
        self.c44 = _safe_divide(self.c44_raw, psi0, "c44 normalization")
        names = ("sigma11", "sigma22", "sigma33", "sigma12", "sigma23", "sigma13")
        self.sigma = tuple(_safe_divide(v, psi0, f"{nm} normalization")
                           for v, nm in zip(self.sigma_raw, names))
        c11, c12, c44 = self.c11, self.c12, self.c44
        den = pow(c11, 2) + c11 * c12 - 2 * pow(c12, 2)
        if den != 0.0 and c44 != 0.0:
            self.s11 = (c11 + c12) / den
            self.s12 = -c12 / den
            self.s44 = 1 / c44
        else:
            # the reference divides by zero here; a config without elastic
            # constants has no use for the compliance
            self.s11 = self.s12 = self.s44 = 0.0
        self.elasC1 = (2 * c44 * (1.5 * self.lambda111 ** 2) - (c11 - c12) * (1.5 * self.lambda100) ** 2)
        self.elasC2 = -1.5 * self.lambda100 * (c11 - c12)
        self.elasC3 = -6.0 * self.lambda111 * c44
        self.dt = _safe_divide(self.timestep * (MU0 * GAMMA) * self.ms, (1 + self.alpha_damp ** 2), "Time step dt")
        self.astar = _safe_divide(2 * self.AA, self.ld ** 2, "Exchange parameter")
        self.alpha = self.astar * self.dt
        self.Hext = tuple(_safe_divide(h, self.ms, f"Hext{i + 1} normalization")
                          for i, h in enumerate(self.Hext_raw))
        self.dHext = tuple(_safe_divide(h, self.ms, f"dHext{i + 1} normalization")
                           for i, h in enumerate(self.dHext_raw))
        return self

    # The LLG step uses zero elastic couplings when ME is off
    # (Micromagnetics.py:40-43).
    @property
    def step_elasC(self):
        if not self.ME:
            return 0.0, 0.0, 0.0
        return self.elasC1, self.elasC2, self.elasC3

    @property
    def alpha1(self) -> float:
        """Exchange weight of the A1 = alpha1 K + M system (assemble_simulation_operators.py:39)."""
        return self.alpha

    @property
    def alpha2(self) -> float:
        """Exchange weight of the A2 system (assemble_simulation_operators.py:40)."""
        return self.alpha * self.alpha_damp

    def with_(self, **kw) -> "SimParams":
        return replace(self, **kw).finalize()


def params_from_config(config: dict, config_path=None, output_dir=None) -> SimParams:
    """Build SimParams from a parsed config dict (schema of parameters.py:59-174)."""
    physics = config["physics"]
    mag = physics["magnetic"]
    p = SimParams()
    p.ms = mag["ms"]
    p.AA_raw = mag["exchange_stiffness"]
    p.K1_raw = mag["anisotropy_k1"]
    el = physics.get("elastic", {}) or {}
    p.c11_raw, p.c12_raw, p.c44_raw = el.get("c11", 0.0), el.get("c12", 0.0), el.get("c44", 0.0)
    ms_ = physics.get("magnetostriction", {}) or {}
    p.lambda100 = ms_.get("lambda100", 0.0)
    p.lambda111 = ms_.get("lambda111", 0.0)
    demag = physics["demagnetization"]
    p.N_x, p.N_y, p.N_z = demag["n_x"], demag["n_y"], demag["n_z"]
    fld = physics["external_field"]
    p.Hext_raw = (fld["hext1"], fld.get("hext2", 0.0), fld.get("hext3", 0.0))
    p.dHext_raw = (fld["dhext1"], fld.get("dhext2", 0.0), fld.get("dhext3", 0.0))
    st = physics.get("external_stress", {}) or {}
    p.sigma_raw = tuple(st.get(k, 0.0) for k in ("sigma11", "sigma22", "sigma33", "sigma12", "sigma23", "sigma13"))
    p.rot111 = bool(physics["rotation_111"])
    p.ME = bool(physics["magnetoelastic_coupling"])
    p.ld = physics["characteristic_length"]

    grid = config["grid"]
    p.grid_type = grid["type"]
    p.defect_center = grid.get("defect_center")
    if p.grid_type == "Hex":
        cm = grid["cubic_mesh"]
        p.Nx, p.Ny, p.Nz = cm.get("nx"), cm.get("ny"), cm.get("nz")
        p.Ndx, p.Ndy, p.Ndz = cm.get("ndx"), cm.get("ndy"), cm.get("ndz")
    elif p.grid_type == "Tet":
        tm = grid["tet_mesh"]
        p.mesh_file = tm["mesh_file"]
        p.defect_shape = tm["defect_shape"]
        p.defect_parameters = tm["defect_parameters"]
        p.defect_rotation = tm.get("rotation_matrix", None)
    else:
        raise NotImplementedError(f"Grid type '{p.grid_type}' is not supported.")

    sim = config["simulation"]
    p.precision = sim["precision"]
    llg = sim["llg"]
    p.timestep = llg["timestep"]
    p.alpha_damp = llg["alpha_damping"]
    p.LLG_accuracy_factor = llg["llg_accuracy_factor"]
    solver = sim["solver"]
    p.tol = solver["tolerance"]
    p.maxiter = solver["max_iterations"]
    p.use_init_factor = solver["initial_factor"]
    p.restart = sim.get("restart", False)
    p.restart_m = sim.get("restart_magnetization", None)
    p.initial_magnetization = None if p.restart else sim.get("initial_magnetization", [1.0, 0.0, 0.0])

    stop = sim["stop_condition"]
    comp = stop.get("component", None)
    if comp is None:
        d = stop.get("direction", None)
        if d is None:
            d = np.array([1.0, 0.0, 0.0])
        else:
            d = np.asarray(d, dtype=np.float64)
            nrm = np.linalg.norm(d)
            if nrm > 0:
                d = d / nrm
            else:
                raise ValueError("Direction vector cannot be zero.")
    else:
        d = np.zeros(3)
        d[comp] = 1.0
    p.stop_direction = tuple(float(v) for v in d)
    sv = stop.get("value", -0.95)
    if not (0 > sv > -1):
        sv = -0.95
    p.stop_value = sv

    out = config.get("output", {}) or {}
    p.write_m = out.get("write_magnetization", True)
    p.save_frequency = int(out.get("save_frequency", 1000))
    p.vtu_alpha = out.get("vtu_blend_alpha", 0.05)
    p.output_dir = str(output_dir) if output_dir is not None else "."
    p.config_path = str(config_path) if config_path is not None else None
    return p.finalize()


def load_parameters(config_path=None) -> SimParams:
    """Load SimParams from a YAML file.

    The path defaults the way the reference resolves it (parameters.py:44-48):
    ``$CUPYMAG_CONFIG_PATH`` or ``config.yaml`` in the working directory.
    """
    if config_path is None:
        config_path = os.environ.get("CUPYMAG_CONFIG_PATH", "config.yaml")
    config_path = Path(config_path).resolve()
    loader = ConfigLoader(config_path)
    return params_from_config(loader.config, config_path=config_path, output_dir=loader.get_output_dir())
