"""Case-file driver: runs the reference's case files on the GPU.

The parser reads the reference's case format (CaseInput::load,
src/CaseInput.cpp: ``key = value`` lines, ``#`` comments, ``boundary
<patch> <kind> <values...>`` lines) for the keys of the solver path --
equation (diffusion, euler, navier_stokes, rans_sa), mesh_file (.fvmesh),
nsteps, gamma, cfl, cfl_mode with the ramp parameters, flux_scheme,
gradient_scheme, mu, prandtl, gas_constant, prandtl_t, initial_nut, the SA
constants, the initial conditions, residual_file / residual_interval, the
per-variable residual tolerances, checkpoint_file, exact Riemann settings,
the diffusion parameters and the force reference quantities.  Keys that
belong to other parts of the reference's program (VTK output, SST, mesh
reports, boundary-layer diagnostics, thread counts) are recorded in
``CaseInput.ignored`` and have no effect.

:func:`run_case` follows the reference's run loop (src/main.cpp run_euler
and its Navier-Stokes / RANS-SA / diffusion siblings): resume from the
checkpoint if it exists, step, stop on a non-finite residual, update the
CFL number with the residual-trend ramp (src/CflRamp.cpp:7-27), write the
residual CSV, stop once every enabled tolerance holds, and write the
checkpoint at the end.

    python -m finitevolume_gb300.case <file.case>
"""
from __future__ import annotations

import dataclasses
import math
import os
import sys
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import io as fvio
from . import solvers as S
from .fvmesh import read_fvmesh


@dataclasses.dataclass
class CflRampParams:
    """CflRampParams (include/CflRamp.h): case keys cfl_min, cfl_ramp_growth,
    cfl_ramp_shrink, cfl_ramp_window, cfl_ramp_divergence_threshold."""
    cfl_min: float = 0.05
    growth_factor: float = 1.5
    shrink_factor: float = 0.5
    window: int = 15
    divergence_threshold: float = 2.0


def next_cfl(current: float, cfl_max: float, history: List[float], params: CflRampParams) -> float:
    """The residual-trend CFL update of src/CflRamp.cpp:7-27: over a full
    window, a rise of more than the divergence threshold (decades) resets
    to cfl_min, a falling trend grows the CFL number, a rise beyond the
    ~10% dead band shrinks it, otherwise it holds; clamped to
    [cfl_min, cfl_max]."""
    if len(history) < params.window:
        return current
    trend = math.log10(history[-1]) - math.log10(history[0])
    dead_band = math.log10(1.1)
    nxt = current
    if trend > params.divergence_threshold:
        nxt = params.cfl_min
    elif trend < 0.0:
        nxt = current * params.growth_factor
    elif trend > dead_band:
        nxt = current * params.shrink_factor
    return min(max(nxt, params.cfl_min), cfl_max)


_IGNORED = {"output_file", "write_interval", "num_threads", "scratch_dir", "output_precision_vtk",
            "resolution_report_file", "resolution_report_interval", "wall_forces_file", "wall_forces_interval",
            "wall_profile_file", "wall_profile_interval", "boundary_layer_max_distance", "boundary_layer_n_samples",
            "boundary_layer_method", "sst_limiter", "sst_kato_launder", "sst_turbulence_intensity",
            "sst_eddy_viscosity_ratio", "initial_k", "initial_omega", "u_adv", "v_adv", "residual_tolerance_k",
            "residual_tolerance_omega", "ransSST_init"}


@dataclasses.dataclass
class CaseInput:
    """The solver-path subset of CaseInput (include/CaseInput.h), with the
    reference's defaults."""
    mesh_file: str = ""
    equation: str = "diffusion"
    nsteps: int = 500
    gamma: float = 1.4
    cfl: float = 0.5
    cfl_mode: str = "fixed"
    cfl_ramp: CflRampParams = dataclasses.field(default_factory=CflRampParams)
    flux_scheme: str = "rusanov"
    gradient_scheme: str = "least-squares"
    exact_riemann_tol: float = 1e-6
    exact_riemann_max_iter: int = 20
    mu: float = 0.0
    prandtl: float = 0.72
    gas_constant: float = 1.0
    prandtl_t: float = 0.9
    initial_nut: float = 0.0
    sa: S.SAModelConstants = dataclasses.field(default_factory=S.SAModelConstants)
    init: Dict[str, Tuple[str, List[float]]] = dataclasses.field(default_factory=dict)
    boundaries: List[Tuple[str, str, List[float]]] = dataclasses.field(default_factory=list)
    residual_file: str = ""
    residual_interval: int = 1
    output_precision: int = 6
    tolerances: Dict[str, float] = dataclasses.field(default_factory=dict)
    checkpoint_file: str = ""
    alpha: float = 0.01
    dt: float = 0.001
    initial_value: float = 1.0
    initial_radius: float = 0.25
    reference: Dict[str, float] = dataclasses.field(default_factory=dict)
    ignored: List[str] = dataclasses.field(default_factory=list)

    @classmethod
    def load(cls, path: str) -> "CaseInput":
        c = cls()
        base = os.path.dirname(os.path.abspath(path))
        with open(path) as f:
            for n, raw in enumerate(f, 1):
                line = raw.split("#", 1)[0].strip()
                if not line:
                    continue
                words = line.split()
                if words[0] == "boundary":
                    if len(words) < 3:
                        raise ValueError(f"{path}:{n}: boundary needs a patch and a kind")
                    c.boundaries.append((words[1], words[2], [float(x) for x in words[3:]]))
                    continue
                if "=" not in line:
                    continue
                key, value = (x.strip() for x in line.split("=", 1))
                c._set(key, value, path, n, base)
        return c

    def _set(self, key, value, path, n, base):
        num = {"gamma", "cfl", "exact_riemann_tol", "mu", "prandtl", "gas_constant", "prandtl_t", "initial_nut",
               "alpha", "dt", "initial_value", "initial_radius"}
        ints = {"nsteps", "residual_interval", "exact_riemann_max_iter", "output_precision"}
        ramp = {"cfl_min": "cfl_min", "cfl_ramp_growth": "growth_factor", "cfl_ramp_shrink": "shrink_factor",
                "cfl_ramp_window": "window", "cfl_ramp_divergence_threshold": "divergence_threshold"}
        refs = {"reference_density", "reference_velocity_x", "reference_velocity_y", "reference_pressure",
                "reference_length", "moment_reference_x", "moment_reference_y"}
        try:
            if key == "mesh_file":
                self.mesh_file = value if os.path.isabs(value) else os.path.join(base, value)
            elif key in num:
                setattr(self, key, float(value))
            elif key in ints:
                setattr(self, key, int(value))
            elif key in ramp:
                setattr(self.cfl_ramp, ramp[key], int(value) if key == "cfl_ramp_window" else float(value))
            elif key.startswith("sa_") and hasattr(self.sa, key[3:]):
                setattr(self.sa, key[3:], float(value))
            elif key in ("equation", "cfl_mode", "flux_scheme", "gradient_scheme"):
                setattr(self, key, value)
            elif key in ("euler_init", "ns_init", "ransSA_init"):
                w = value.split()
                self.init[key] = (w[0], [float(x) for x in w[1:]])
            elif key == "residual_file":
                self.residual_file = value if (not value or os.path.isabs(value)) else os.path.join(base, value)
            elif key == "checkpoint_file":
                self.checkpoint_file = value if (not value or os.path.isabs(value)) else os.path.join(base, value)
            elif key.startswith("residual_tolerance"):
                self.tolerances[key[len("residual_tolerance"):].lstrip("_") or "phi"] = float(value)
            elif key in refs:
                self.reference[key] = float(value)
            else:
                self.ignored.append(key)
        except ValueError as e:
            raise ValueError(f"{path}:{n}: key '{key}': {e}") from None


def _ic(c: CaseInput, key: str) -> S.EulerInitialCondition:
    mode, v = c.init.get(key, ("freestream", [1.0, 0.0, 0.0, 1.0]))
    if mode == "tworegion":
        return S.EulerInitialCondition(S.EulerICMode.TwoRegion, rho_l=v[0], u_l=v[1], v_l=v[2], p_l=v[3], rho_r=v[4],
                                       u_r=v[5], v_r=v[6], p_r=v[7], x0=v[8])
    return S.EulerInitialCondition(S.EulerICMode.Freestream, rho=v[0], u=v[1], v=v[2], p=v[3])


_FLUX = {"rusanov": S.NumericalFluxScheme.Rusanov, "hllc": S.NumericalFluxScheme.HLLC,
         "exact": S.NumericalFluxScheme.Exact}
_GRAD = {"least-squares": S.GradientScheme.LeastSquares, "green-gauss": S.GradientScheme.GreenGauss}


def _bc_map(c: CaseInput, names: List[str]):
    found = {p: (kind, vals) for p, kind, vals in c.boundaries}
    unknown = [p for p in found if p not in names]
    if unknown:
        raise ValueError(f"boundary condition for unknown patch(es) {unknown}")
    return found


def build_solver(c: CaseInput, mesh: "S.Mesh"):
    names = mesh.patch_names
    bmap = _bc_map(c, names)
    flux, grad = _FLUX[c.flux_scheme], _GRAD[c.gradient_scheme]
    if c.equation == "euler":
        bcs = []
        for n in names:
            kind, v = bmap.get(n, ("wall", []))
            if kind == "farfield":
                bcs.append(S.EulerBoundaryCondition(S.EulerBoundaryType.Farfield, S.from_primitive(*v[:4], c.gamma)))
            elif kind == "outflow":
                bcs.append(S.EulerBoundaryCondition(S.EulerBoundaryType.Outflow))
            else:
                bcs.append(S.EulerBoundaryCondition(S.EulerBoundaryType.Wall))
        return S.EulerFVMSolver(mesh, bcs, c.gamma, c.cfl, _ic(c, "euler_init"), flux, c.exact_riemann_tol,
                                c.exact_riemann_max_iter)
    if c.equation in ("navier_stokes", "rans_sa"):
        pre = "ns_" if c.equation == "navier_stokes" else "ransSA_"
        out = []
        for n in names:
            kind, v = bmap.get(n, (pre + "wall", []))
            k = kind[len(pre):] if kind.startswith(pre) else kind
            b = S.NSBoundaryCondition(S.NSBoundaryType.NoSlipWall)
            nut = 0.0
            if k == "wall_isothermal":
                b.is_isothermal_wall, b.wall_temperature = True, v[0]
            elif k == "wall_moving":
                b.wall_u, b.wall_v = v[0], v[1]
            elif k == "wall_moving_isothermal":
                b.wall_u, b.wall_v, b.is_isothermal_wall, b.wall_temperature = v[0], v[1], True, v[2]
            elif k == "outflow":
                b = S.NSBoundaryCondition(S.NSBoundaryType.Outflow)
            elif k == "farfield":
                b = S.NSBoundaryCondition(S.NSBoundaryType.Farfield,
                                          farfield_state=list(S.from_primitive(*v[:4], c.gamma)))
                nut = v[4] if len(v) > 4 else 0.0
            out.append(b if c.equation == "navier_stokes" else S.RANSBoundaryConditionSA(b, nut))
        if c.equation == "navier_stokes":
            return S.NavierStokesFVMSolver(mesh, out, c.gamma, c.gas_constant, c.mu, c.prandtl, c.cfl,
                                           _ic(c, "ns_init"), flux, grad, c.exact_riemann_tol, c.exact_riemann_max_iter)
        return S.RANSTurbulenceSASolver(mesh, out, c.gamma, c.gas_constant, c.mu, c.prandtl, c.prandtl_t, c.cfl,
                                        _ic(c, "ransSA_init"), c.initial_nut, flux, grad, c.exact_riemann_tol,
                                        c.exact_riemann_max_iter, c.sa)
    if c.equation == "diffusion":
        kinds = {"dirichlet": S.BoundaryType.Dirichlet, "neumann": S.BoundaryType.Neumann}
        patches = {n: (kinds[k], v[0] if v else 0.0) for n, (k, v) in bmap.items()}
        return S.UnstructuredFVMSolver(mesh, c.alpha, c.dt, c.initial_value, c.initial_radius, patches)
    raise ValueError(f"equation '{c.equation}' is not on the GPU path (diffusion, euler, navier_stokes, rans_sa)")


def run_case(c: CaseInput, mesh: Optional["S.Mesh"] = None, log=print) -> dict:
    """Run a loaded case on the GPU; returns the outcome."""
    if mesh is None:
        if not c.mesh_file.endswith(".fvmesh"):
            raise ValueError("mesh_file: only .fvmesh meshes are read (Gmsh .msh is not on the GPU path)")
        mesh = S.Mesh(read_fvmesh(c.mesh_file))
    solver = build_solver(c, mesh)
    flow = c.equation != "diffusion"
    rans = c.equation == "rans_sa"
    eq_name = {"euler": "euler", "navier_stokes": "navier_stokes", "rans_sa": "rans_sa"}.get(c.equation, "diffusion")
    cur_cfl = c.cfl
    hist: List[float] = []
    if flow and c.cfl_mode == "ramp":
        cur_cfl = c.cfl_ramp.cfl_min
        solver.set_cfl(cur_cfl)
    start = 1
    if c.checkpoint_file and os.path.exists(c.checkpoint_file):
        if flow:
            if rans:
                try:
                    payload, step, _ = fvio.read_checkpoint(c.checkpoint_file, "rans_sa", mesh.n_cells)
                    solver.set_field(np.ascontiguousarray(payload[:, :4]), np.ascontiguousarray(payload[:, 4]))
                except Exception:
                    payload, step, _ = fvio.read_checkpoint(c.checkpoint_file, None, mesh.n_cells)
                    solver.set_field(payload)
            else:
                payload, step, _ = fvio.read_checkpoint(c.checkpoint_file, None, mesh.n_cells)
                solver.set_field(payload)
        else:
            payload, step, _ = fvio.read_checkpoint(c.checkpoint_file, "diffusion", mesh.n_cells)
            solver.set_field(payload)
        start = step + 1
        log(f"Resuming from checkpoint at step {step}")
    csv = None
    if c.residual_file:
        os.makedirs(os.path.dirname(os.path.abspath(c.residual_file)), exist_ok=True)
        if flow:
            csv = fvio.ResidualCSV(c.residual_file, c.residual_interval, c.output_precision,
                                   extra=("nut",) if rans else ())
        else:
            csv = open(c.residual_file, "w")
            csv.write("step,residual\n")
    tol = c.tolerances
    outcome, last = "completed", start - 1
    for k in range(start, c.nsteps + 1):
        solver.step()
        last = k
        if flow:
            r = solver.residual().as_array()
            vals = list(r) + ([solver.nut_residual()] if rans else [])
        else:
            vals = [solver.residual_norm()]
        if not all(np.isfinite(vals)):
            outcome = "diverged"
            break
        if flow and c.cfl_mode == "ramp":
            hist.append(vals[0])
            if len(hist) > c.cfl_ramp.window:
                hist.pop(0)
            cur_cfl = next_cfl(cur_cfl, c.cfl, hist, c.cfl_ramp)
            solver.set_cfl(cur_cfl)
        if csv is not None:
            if flow:
                csv.record(k, vals)
            elif k % max(1, c.residual_interval) == 0:
                csv.write(f"{k},{vals[0]:.{c.output_precision}g}\n")
                csv.flush()
        if tol:
            names = ["rho", "rho_u", "rho_v", "E", "nut"] if flow else ["phi"]
            checks = [(vals[i] < tol[nm]) for i, nm in enumerate(names[:len(vals)]) if nm in tol]
            if checks and all(checks):
                outcome = "converged"
                break
    if csv is not None:
        csv.close()
    if c.checkpoint_file and last >= start and outcome != "diverged":
        os.makedirs(os.path.dirname(os.path.abspath(c.checkpoint_file)), exist_ok=True)
        if rans:
            payload = np.concatenate([solver.field(), solver.nut_field()[:, None]], 1)
        elif flow:
            payload = solver.field()
        else:
            payload = solver.field()
        fvio.write_checkpoint(c.checkpoint_file, eq_name, last, payload)
    res = {"outcome": outcome, "last_step": last, "cfl": cur_cfl}
    if flow:
        res["residual"] = solver.residual().as_array().tolist()
        if rans:
            res["residual_nut"] = solver.nut_residual()
    return res


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 1:
        print("usage: python -m finitevolume_gb300.case <file.case>", file=sys.stderr)
        return 2
    c = CaseInput.load(argv[0])
    if c.ignored:
        print(f"note: keys outside the GPU solver path ignored: {', '.join(sorted(set(c.ignored)))}", file=sys.stderr)
    res = run_case(c)
    print(res)
    return 0 if res["outcome"] != "diverged" else 1


if __name__ == "__main__":
    sys.exit(main())
