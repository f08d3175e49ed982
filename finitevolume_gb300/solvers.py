"""Python mirror of the reference's solver interface over the C ABI.

Names, argument order and meaning follow the reference classes so that code
written against them reads the same:

* ``EulerFVMSolver(mesh, boundary_conditions, gamma, cfl, initial_condition,
  flux_scheme, exact_riemann_tol, exact_riemann_max_iter)`` with ``step``,
  ``run``, ``field``, ``residual``, ``set_field``, ``set_cfl``, ``gas_gamma``
  (include/EulerFVMSolver.h:107-160).
* ``EulerBoundaryType`` / ``EulerBoundaryCondition`` / ``EulerICMode`` /
  ``EulerInitialCondition`` / ``NumericalFluxScheme`` /
  ``EulerResidualNorms`` (include/EulerFVMSolver.h:17-67).

All arithmetic runs in the CUDA library; these classes only marshal arrays.
Extensions beyond the reference (second order, SSP-RK3, local time
stepping, characteristic farfield, FP32 flux, strict IEEE mode) are keyword
arguments with reference-mode defaults.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import enum
from typing import Optional, Sequence

import numpy as np

from . import capi
from .fvmesh import PolyMesh


class EulerBoundaryType(enum.IntEnum):
    Wall = 0
    Farfield = 1
    Outflow = 2
    CharacteristicFarfield = 3  # extension: Riemann-invariant farfield


class NumericalFluxScheme(enum.IntEnum):
    Rusanov = 0
    HLLC = 1
    Exact = 2


class EulerICMode(enum.IntEnum):
    Freestream = 0
    TwoRegion = 1


class GradientScheme(enum.IntEnum):
    LeastSquares = 0
    GreenGauss = 1


class Limiter(enum.IntEnum):
    NoLimiter = 0
    BarthJespersen = 1
    Venkatakrishnan = 2


def from_primitive(rho: float, u: float, v: float, p: float, gamma: float) -> np.ndarray:
    """Conserved state from primitives, E = p/(g-1) + rho (u^2+v^2)/2 (EulerState.h:45-52)."""
    return np.array([rho, rho * u, rho * v, p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)])


@dataclasses.dataclass
class EulerBoundaryCondition:
    type: EulerBoundaryType = EulerBoundaryType.Wall
    farfield_state: Sequence[float] = (0.0, 0.0, 0.0, 0.0)  # conserved


@dataclasses.dataclass
class EulerInitialCondition:
    mode: EulerICMode = EulerICMode.Freestream
    rho: float = 1.0
    u: float = 0.0
    v: float = 0.0
    p: float = 1.0
    rho_l: float = 1.0
    u_l: float = 0.0
    v_l: float = 0.0
    p_l: float = 1.0
    rho_r: float = 0.125
    u_r: float = 0.0
    v_r: float = 0.0
    p_r: float = 0.1
    x0: float = 0.0


@dataclasses.dataclass
class EulerResidualNorms:
    rho: float = 0.0
    rho_u: float = 0.0
    rho_v: float = 0.0
    E: float = 0.0

    def as_array(self) -> np.ndarray:
        return np.array([self.rho, self.rho_u, self.rho_v, self.E])


class Mesh:
    """Device-ready mesh built by the library from a :class:`PolyMesh`.

    Topology follows the reference reader (first visitor owns each face);
    ``reorder`` chooses the device cell order ("morton", "rcm" or "none").
    """

    def __init__(self, poly: PolyMesh, reorder: str = "morton"):
        L = capi.lib()
        h = C.c_void_p()
        nodes = np.ascontiguousarray(poly.nodes, dtype=np.float64)
        off = np.ascontiguousarray(poly.cell_off, dtype=np.int64)
        cn = np.ascontiguousarray(poly.cell_nodes, dtype=np.int32)
        be = np.ascontiguousarray(poly.bedges, dtype=np.int32)
        bp = np.ascontiguousarray(poly.bpatch, dtype=np.int32)
        capi.check(L.fv_mesh_create_polygons(nodes.shape[0], capi.dptr(nodes), poly.n_cells, capi.i64ptr(off),
                                             capi.i32ptr(cn), be.shape[0], capi.i32ptr(be), capi.i32ptr(bp),
                                             len(poly.patch_names), capi.REORDER[reorder], C.byref(h)))
        self._h = h
        self.poly = poly
        self.patch_names = list(poly.patch_names)
        cnt = np.zeros(5, dtype=np.int64)
        capi.check(L.fv_mesh_counts(h, capi.i64ptr(cnt)))
        self.n_cells, self.n_faces, self.n_bfaces, self.n_patches, self.n_entries = (int(x) for x in cnt)

    @property
    def handle(self):
        return self._h

    def export(self):
        """Reference-numbered topology: dict of numpy arrays."""
        F, N = self.n_faces, self.n_cells
        fi = np.zeros((F, 5), np.int32)
        fd = np.zeros((F, 5), np.float64)
        cd = np.zeros((N, 3), np.float64)
        off = np.zeros(N + 1, np.int32)
        cf = np.zeros(self.n_entries, np.int32)
        capi.check(capi.lib().fv_mesh_export(self._h, capi.i32ptr(fi), capi.dptr(fd), capi.dptr(cd),
                                             capi.i32ptr(off), capi.i32ptr(cf)))
        return {"faces_i32": fi, "faces_f64": fd, "cells_f64": cd, "cell_face_off": off, "cell_faces": cf}

    def dataflow_plan(self, patch_types, blocks: int = 152) -> dict:
        """The partition of the persistent first-order kernel's dataflow form
        over ``blocks`` blocks (one per SM; host side, for inspection):
        device-numbered ``cell_off``, ``face_off``, ``faces``, the dependency
        lists ``dep_face``/``dep_cell`` with their offsets, ``face_cells``
        (left, right of each face), ``nb`` and ``used`` (False when a block
        would wait for more than 32 blocks in a phase)."""
        pt = np.ascontiguousarray(patch_types, dtype=np.int32)
        if pt.shape[0] < self.n_patches:
            raise ValueError("one boundary type per patch")
        cnt = np.zeros(4, np.int32)
        null = C.POINTER(C.c_int32)()
        L = capi.lib()
        capi.check(L.fv_mesh_dataflow_plan(self._h, capi.i32ptr(pt), int(blocks), capi.i32ptr(cnt), null, null, null,
                                           null, null, null, null, null))
        nb, nd1, nd2 = int(cnt[0]), int(cnt[1]), int(cnt[2])
        out = {"cell_off": np.zeros(nb + 1, np.int32), "face_off": np.zeros(nb + 1, np.int32),
               "faces": np.zeros(self.n_faces, np.int32), "dep_face_off": np.zeros(nb + 1, np.int32),
               "dep_face": np.zeros(max(nd1, 1), np.int32), "dep_cell_off": np.zeros(nb + 1, np.int32),
               "dep_cell": np.zeros(max(nd2, 1), np.int32), "face_cells": np.zeros((self.n_faces, 2), np.int32)}
        capi.check(L.fv_mesh_dataflow_plan(self._h, capi.i32ptr(pt), int(blocks), capi.i32ptr(cnt),
                                           *(capi.i32ptr(out[k]) for k in ("cell_off", "face_off", "faces",
                                                                            "dep_face_off", "dep_face",
                                                                            "dep_cell_off", "dep_cell",
                                                                            "face_cells"))))
        out["dep_face"] = out["dep_face"][:nd1]
        out["dep_cell"] = out["dep_cell"][:nd2]
        out["nb"] = nb
        out["used"] = bool(cnt[3])
        return out

    def permutation(self) -> np.ndarray:
        p = np.zeros(self.n_cells, np.int32)
        capi.check(capi.lib().fv_mesh_permutation(self._h, capi.i32ptr(p)))
        return p

    def agglomerate(self):
        """The first coarse level multigrid builds from this mesh (host
        side): dict with ``agg`` (agglomerate of each fine cell), coarse
        ``cells_f64`` (volume, cx, cy), ``faces_i32`` (left, right, patch)
        and ``faces_f64`` (nx, ny, length)."""
        n = np.zeros(2, np.int32)
        null = C.POINTER(C.c_int32)()
        dnull = C.POINTER(C.c_double)()
        capi.check(capi.lib().fv_mesh_agglomerate(self._h, capi.i32ptr(n), null, dnull, null, dnull))
        nc, nf = int(n[0]), int(n[1])
        agg = np.zeros(self.n_cells, np.int32)
        cd = np.zeros((nc, 3), np.float64)
        fi = np.zeros((nf, 3), np.int32)
        fd = np.zeros((nf, 3), np.float64)
        capi.check(capi.lib().fv_mesh_agglomerate(self._h, capi.i32ptr(n), capi.i32ptr(agg), capi.dptr(cd),
                                                  capi.i32ptr(fi), capi.dptr(fd)))
        return {"agg": agg, "cells_f64": cd, "faces_i32": fi, "faces_f64": fd}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                capi.lib().fv_mesh_destroy(h)
            except Exception:
                pass
            self._h = None


def _bc_array(bcs: Sequence[EulerBoundaryCondition]):
    arr = (capi.BC * max(1, len(bcs)))()
    for i, b in enumerate(bcs):
        arr[i].type = int(b.type)
        for k in range(4):
            arr[i].state[k] = float(b.farfield_state[k])
    return arr


def _ic_struct(ic: EulerInitialCondition) -> capi.IC:
    s = capi.IC()
    s.two_region = 1 if ic.mode == EulerICMode.TwoRegion else 0
    for f in ("rho", "u", "v", "p", "rho_l", "u_l", "v_l", "p_l", "rho_r", "u_r", "v_r", "p_r", "x0"):
        setattr(s, f, float(getattr(ic, f)))
    return s


def _launch_cache_path() -> str:
    import os
    root = os.environ.get("FV_MESH_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "finitevolume_gb300"))
    return os.path.join(root, "launch_shapes.json")


def _autotune(handle, key: str, steps: int, cache: bool) -> dict:
    """Launch shapes from the cache, or tuned on this solver and cached."""
    import json
    import os
    path = _launch_cache_path()
    table = {}
    if cache and os.path.exists(path):
        try:
            with open(path) as f:
                table = json.load(f)
        except (OSError, ValueError):
            table = {}
    if cache and key in table:
        b = np.array(table[key], dtype=np.int32)
        capi.check(capi.lib().fv_solver_set_launch(handle, capi.i32ptr(b)))
        return {"gradients": int(b[0]), "faces": int(b[1]), "cells": int(b[2]), "cached": True}
    b = np.zeros(3, np.int32)
    capi.check(capi.lib().fv_solver_autotune(handle, int(steps), capi.i32ptr(b)))
    if cache:
        table[key] = b.tolist()
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + f".{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(table, f)
        os.replace(tmp, path)
    return {"gradients": int(b[0]), "faces": int(b[1]), "cells": int(b[2]), "cached": False}


def _shape_key(o, n_cells: int, batch: bool) -> str:
    return (f"p{o.precision}-o{o.order}-f{o.flux}-g{o.gradient}-l{o.limiter}-rk{o.rk_stages}-dt{o.dt_mode}"
            f"-b{int(batch)}-n{int(np.log2(max(n_cells, 1)))}")


class EulerFVMSolver:
    """GPU explicit Euler solver with the reference's constructor and methods."""

    def __init__(self, input_mesh: Mesh, boundary_conditions: Sequence[EulerBoundaryCondition], gamma: float,
                 cfl: float, initial_condition: EulerInitialCondition,
                 flux_scheme: NumericalFluxScheme = NumericalFluxScheme.Rusanov, exact_riemann_tol: float = 1e-6,
                 exact_riemann_max_iter: int = 20, *, order: int = 1, rk_stages: int = 1, local_dt: bool = False,
                 gradient: GradientScheme = GradientScheme.LeastSquares, limiter: Limiter = Limiter.Venkatakrishnan,
                 venkat_k: float = 5.0, fp32_flux: bool = False, strict: bool = False, _viscous=None, _rans=None):
        if not isinstance(input_mesh, Mesh):
            input_mesh = Mesh(input_mesh)
        self.mesh = input_mesh
        L = capi.lib()
        o = capi.default_options()
        if _viscous is not None:
            o.viscous = 1
            o.gas_constant, o.mu, o.prandtl = (float(x) for x in _viscous)
        if _rans is not None:
            o.viscous = 2
            o.prandtl_t = float(_rans["prandtl_t"])
            o.initial_nut = float(_rans["initial_nut"])
            for i, v in enumerate(_rans["sa"]):
                o.sa[i] = float(v)
        o.flux = int(flux_scheme)
        o.exact_tol = float(exact_riemann_tol)
        o.exact_max_iter = int(exact_riemann_max_iter)
        o.order = int(order)
        o.rk_stages = int(rk_stages)
        o.dt_mode = 1 if local_dt else 0
        o.gradient = int(gradient)
        o.limiter = int(limiter)
        o.venkat_k = float(venkat_k)
        o.precision = 1 if fp32_flux else 0
        o.strict = 1 if strict else 0
        self._opt = o
        bc = boundary_conditions if isinstance(boundary_conditions, C.Array) else _bc_array(boundary_conditions)
        ic = _ic_struct(initial_condition)
        h = C.c_void_p()
        capi.check(L.fv_solver_create(input_mesh.handle, bc, len(boundary_conditions), float(gamma), float(cfl),
                                      C.byref(ic), C.byref(o), C.byref(h)))
        self._h = h
        self.n_cells = input_mesh.n_cells

    # -- reference API -----------------------------------------------------
    def step(self) -> None:
        capi.check(capi.lib().fv_step(self._h, 1, None))

    def run(self, total_steps: int, history: bool = False) -> Optional[np.ndarray]:
        """Advance ``total_steps`` steps; optionally return the n x 4 norm history."""
        if history:
            out = np.zeros((total_steps, 4))
            capi.check(capi.lib().fv_step(self._h, total_steps, capi.dptr(out)))
            return out
        capi.check(capi.lib().fv_step(self._h, total_steps, None))
        return None

    def field(self) -> np.ndarray:
        out = np.zeros((self.n_cells, 4))
        capi.check(capi.lib().fv_get_field(self._h, capi.dptr(out)))
        return out

    def set_field(self, new_U: np.ndarray) -> None:
        u = np.ascontiguousarray(new_U, dtype=np.float64)
        if u.shape != (self.n_cells, 4):
            raise ValueError(f"set_field expects shape {(self.n_cells, 4)}, got {u.shape}")
        capi.check(capi.lib().fv_set_field(self._h, capi.dptr(u)))

    def residual(self) -> EulerResidualNorms:
        out = np.zeros(4)
        capi.check(capi.lib().fv_get_residual(self._h, capi.dptr(out)))
        return EulerResidualNorms(*out.tolist())

    def set_cfl(self, new_cfl: float) -> None:
        capi.check(capi.lib().fv_set_cfl(self._h, float(new_cfl)))

    def gas_gamma(self) -> float:
        g = C.c_double()
        capi.check(capi.lib().fv_get_gamma(self._h, C.byref(g)))
        return g.value

    # -- extensions ----------------------------------------------------------
    def set_launch(self, gradients: int, faces: int, cells: int) -> None:
        """Threads per block of the gradient, face and cell kernels."""
        b = np.array([gradients, faces, cells], np.int32)
        capi.check(capi.lib().fv_solver_set_launch(self._h, capi.i32ptr(b)))

    def multigrid(self, levels: int = 4, smooth: int = 1, relax: float = 0.7) -> None:
        """Agglomeration multigrid V-cycles (steady solves, local dt): each
        step becomes one smoothing iteration plus one V-cycle."""
        capi.check(capi.lib().fv_solver_multigrid(self._h, self.mesh.handle, int(levels), int(smooth), float(relax)))

    def newton(self, max_newton: int = 200, tol: float = 1e-11, limiter_mode: int = 0, **kw):
        """Newton-Krylov steady solve from the current state (pseudo-transient
        continuation, exact Jacobian-vector products, block-Jacobi
        preconditioned GMRES).  ``limiter_mode`` 0 frozen / 1 full limiter
        Jacobian; other keywords: cfl0, cfl_max, cfl_growth, krylov_dim,
        krylov_rtol, precond_sweeps, precond_kind (2 multicolour symmetric
        Gauss-Seidel on FP32 blocks, 1 the same in FP64, 0 block Jacobi),
        max_rel_change.  Returns (history
        [(steps + 1) x 8]: four residual norms, CFL, GMRES iterations, GMRES
        relative residual, step length; Newton steps taken)."""
        o = capi.NewtonOpts()
        capi.lib().fv_newton_default(C.byref(o))
        o.max_newton, o.tol, o.limiter_mode = int(max_newton), float(tol), int(limiter_mode)
        for k, v in kw.items():
            if not hasattr(o, k):
                raise TypeError(f"unknown Newton option {k}")
            setattr(o, k, type(getattr(o, k))(v))
        hist = np.zeros((int(max_newton) + 1, 8))
        it = C.c_int32()
        steps = np.zeros(max(1, getattr(self, "n_instances", 1)), np.int32)
        capi.check(capi.lib().fv_steady_newton(self._h, C.byref(o), capi.dptr(hist), C.byref(it), capi.i32ptr(steps)))
        self.last_newton_instance_steps = steps
        return hist[:it.value + 1], it.value

    def set_persistent(self, on=True) -> None:
        """First-order forward-Euler FP64 path: one persistent cooperative
        launch per chunk of steps (on, the default where supported; with
        local dt in its dataflow form), two kernels per step (off), or
        ``"barrier"`` for the grid-barrier form of the persistent kernel."""
        mode = 2 if on == "barrier" else (1 if on else 0)
        capi.check(capi.lib().fv_solver_set_persistent(self._h, mode))

    def persistent(self):
        """(form in use, grid size in blocks) of the persistent kernel: form
        0 two-kernel path, 1 grid-barrier form, 2 dataflow form."""
        on, grid = C.c_int32(), C.c_int32()
        capi.check(capi.lib().fv_solver_persistent(self._h, C.byref(on), C.byref(grid)))
        return int(on.value), int(grid.value)

    def set_wait_limit(self, cycles: int, phantom_arrivals: int = 0) -> None:
        """Bound (SM clock cycles) on each wait of the persistent kernel
        (grid barrier or neighbour progress); phantom_arrivals > 0 makes
        every grid barrier wait for arrivals that never come (checks the
        FV_ERR_TIMEOUT path)."""
        capi.check(capi.lib().fv_solver_set_wait_limit(self._h, int(cycles), int(phantom_arrivals)))

    def freeze_limiter(self, on: bool = True) -> None:
        """Capture the limiter values at the current state and reuse them in
        every later step (on=False: evaluate the limiter again)."""
        capi.check(capi.lib().fv_solver_freeze_limiter(self._h, 1 if on else 0))

    def limiter_values(self) -> np.ndarray:
        """The frozen limiter values [n_cells, 4] (rho, u, v, p)."""
        out = np.zeros((self.mesh.n_cells, 4))
        capi.check(capi.lib().fv_solver_limiter_values(self._h, capi.dptr(out), None))
        return out

    def set_limiter_values(self, psi) -> None:
        """Freeze the limiter at the given values [n_cells, 4]."""
        capi.check(capi.lib().fv_solver_limiter_values(self._h, None,
                                                       capi.dptr(np.ascontiguousarray(psi, dtype=np.float64))))

    def update_nodes(self, nodes) -> None:
        """Move the mesh nodes ([n_nodes, 2]) and recompute the geometry on
        the device (the state is kept)."""
        xy = np.ascontiguousarray(nodes, dtype=np.float64)
        capi.check(capi.lib().fv_solver_update_nodes(self._h, self.mesh.handle, capi.dptr(xy)))

    def autotune(self, steps: int = 5, cache: bool = True) -> dict:
        """Pick the launch shapes by timing (state preserved); results are
        cached per scheme and mesh-size octave."""
        return _autotune(self._h, _shape_key(self._opt, self.n_cells, False), steps, cache)

    def step_async(self, n: int) -> None:
        capi.check(capi.lib().fv_step_async(self._h, int(n)))

    def step_timed(self, n: int):
        """Advance n steps with per-kernel CUDA-event timing.

        Returns (ms[3], launches[3]) for kernel classes gradients, face fluxes,
        cell update."""
        ms = np.zeros(3)
        cnt = np.zeros(3, np.int32)
        capi.check(capi.lib().fv_step_timed(self._h, int(n), capi.dptr(ms), capi.i32ptr(cnt)))
        return ms, cnt

    def history(self, n: int) -> np.ndarray:
        out = np.zeros((n, 4))
        capi.check(capi.lib().fv_get_history(self._h, int(n), capi.dptr(out)))
        return out

    def set_stream(self, stream_handle: int) -> None:
        capi.check(capi.lib().fv_solver_set_stream(self._h, C.c_void_p(stream_handle)))

    def device_state(self):
        u = C.c_void_p()
        s = C.c_void_p()
        capi.check(capi.lib().fv_device_state(self._h, C.byref(u), C.byref(s)))
        return u.value, s.value

    def wall_forces(self, rho_ref=1.0, u_ref=1.0, v_ref=0.0, p_ref=0.0, length_ref=1.0, moment_x=0.25,
                    moment_y=0.0) -> dict:
        ref = np.array([rho_ref, u_ref, v_ref, p_ref, length_ref, moment_x, moment_y], dtype=np.float64)
        out = np.zeros(11)
        capi.check(capi.lib().fv_wall_forces(self._h, capi.dptr(ref), capi.dptr(out)))
        keys = ["friction_drag", "pressure_drag", "total_drag", "lift", "moment", "cd_friction", "cd_pressure",
                "cd_total", "cl", "cm", "n_wall_faces"]
        return dict(zip(keys, out.tolist()))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                capi.lib().fv_solver_destroy(h)
            except Exception:
                pass
            self._h = None


class BoundaryType(enum.IntEnum):
    """Diffusion boundary kinds (include/UnstructuredMesh.h:49-52)."""
    Dirichlet = 0
    Neumann = 1


_MAX_PATCHES = 32  # boundary-condition table size of the C ABI


class Objective(enum.IntEnum):
    """Wall-force coefficients the adjoint differentiates."""
    Drag = 0
    Lift = 1
    Moment = 2


def force_gradient(solver: "EulerFVMSolver", objective: Objective, ref) -> tuple:
    """(J, dJ/dU [N, 4]) of a pressure force coefficient at the solver's state."""
    r = np.ascontiguousarray(ref, dtype=np.float64)
    val = C.c_double()
    g = np.zeros((solver.n_cells, 4))
    capi.check(capi.lib().fv_force_gradient(solver._h, int(objective), capi.dptr(r), C.byref(val), capi.dptr(g)))
    return val.value, g


class DiscreteAdjoint:
    """Forward/backward pair of the Euler residual R(U, fs) and its adjoint.

    ``forward(U)`` linearises at U (default: the solver's state) and returns
    R(U); ``jvp`` and ``vjp`` are the tangent and cotangent maps at that
    state (limiter values frozen, or differentiated with
    ``full_limiter=True``); ``solve`` returns the adjoint lambda of
    (dR/dU)^T lambda = dJ/dU and fsbar = (dR/dfs)^T lambda, fs being each
    patch's primitive freestream (rho, u, v, p).
    """

    def __init__(self, solver: "EulerFVMSolver", full_limiter: bool = False):
        self.solver = solver
        self.n = solver.n_cells
        self.n_patches = len(solver.mesh.patch_names)
        h = C.c_void_p()
        capi.check(capi.lib().fv_adjoint_create(solver._h, 1 if full_limiter else 0, C.byref(h)))
        self._h = h

    def forward(self, U=None) -> np.ndarray:
        R = np.zeros((self.n, 4))
        u = None if U is None else capi.dptr(np.ascontiguousarray(U, dtype=np.float64))
        capi.check(capi.lib().fv_residual_forward(self._h, u, capi.dptr(R)))
        return R

    def jvp(self, dU, dfs=None) -> np.ndarray:
        dR = np.zeros((self.n, 4))
        d = None
        if dfs is not None:
            pad = np.zeros((_MAX_PATCHES, 4))
            q = np.asarray(dfs, dtype=np.float64).reshape(-1, 4)
            pad[:q.shape[0]] = q
            d = capi.dptr(pad)
        capi.check(capi.lib().fv_residual_jvp(self._h, capi.dptr(np.ascontiguousarray(dU, dtype=np.float64)), d,
                                              capi.dptr(dR)))
        return dR

    def vjp(self, Rbar):
        Ub = np.zeros((self.n, 4))
        fb = np.zeros((_MAX_PATCHES, 4))
        capi.check(capi.lib().fv_residual_backward(self._h, capi.dptr(np.ascontiguousarray(Rbar, dtype=np.float64)),
                                                   capi.dptr(Ub), capi.dptr(fb)))
        return Ub, fb[:self.n_patches]

    # method "krylov": pseudo-time CFL number and preconditioner sweeps
    krylov_cfl = 3e3
    krylov_sweeps = 8

    def solve(self, dJdU, max_iter: int = 20000, tol: float = 1e-12, method: str = "rk", restart: int = 40):
        """Solve (dR/dU)^T lambda = dJdU.  method "rk": SSP-RK3 pseudo-time
        iteration until every residual-norm component is below tol (history
        [iterations, 4] of those norms); "gmres": GMRES(restart) on the
        fixed point of that iteration until its residual falls by the
        factor tol, max_iter matvecs (history [matvecs] of the relative
        GMRES residual); "krylov": pseudo-transient outer iterations on
        the transposed Newton system at CFL ``krylov_cfl``, each one
        GMRES(restart) cycle preconditioned by ``krylov_sweeps`` Gauss-Seidel
        sweeps of the transposed first-order Jacobian, until the adjoint
        residual falls by the factor tol, max_iter matvecs (history:
        relative residual per outer iteration).  Returns lambda, fsbar, history, iterations; the
        final residual norms are kept in ``last_residual`` for "gmres"."""
        lam = np.zeros((self.n, 4))
        fb = np.zeros((_MAX_PATCHES, 4))
        it = C.c_int32()
        g = np.ascontiguousarray(dJdU, dtype=np.float64)
        if method == "gmres":
            hist = np.zeros(max(max_iter, 1))
            res = np.zeros(4)
            capi.check(capi.lib().fv_adjoint_solve_gmres(self._h, capi.dptr(g), int(restart), int(max_iter),
                                                         float(tol), capi.dptr(lam), capi.dptr(fb), capi.dptr(hist),
                                                         C.byref(it), capi.dptr(res)))
            self.last_residual = res
            return lam, fb[:self.n_patches], hist[:it.value], it.value
        if method == "krylov":
            hist = np.zeros(max(max_iter // 2 + 2, 1))
            res = np.zeros(4)
            capi.check(capi.lib().fv_adjoint_solve_krylov(self._h, capi.dptr(g), float(self.krylov_cfl), int(restart),
                                                          int(max_iter), float(tol), int(self.krylov_sweeps),
                                                          capi.dptr(lam), capi.dptr(fb), capi.dptr(hist),
                                                          C.byref(it), capi.dptr(res)))
            self.last_residual = res
            n_cycles = int(np.count_nonzero(hist))
            return lam, fb[:self.n_patches], hist[:n_cycles], it.value
        if method != "rk":
            raise ValueError("method: 'rk', 'gmres' or 'krylov'")
        hist = np.zeros((max(max_iter, 1), 4))
        capi.check(capi.lib().fv_adjoint_solve(self._h, capi.dptr(g), int(max_iter), float(tol), capi.dptr(lam),
                                               capi.dptr(fb), capi.dptr(hist), C.byref(it)))
        self.last_residual = hist[it.value - 1] if it.value else None
        return lam, fb[:self.n_patches], hist[:it.value], it.value

    def shape_gradient(self, objective: Objective, ref) -> np.ndarray:
        """dJ/dX [n_nodes, 2] of the objective the last ``solve`` used."""
        r = np.ascontiguousarray(ref, dtype=np.float64)
        out = np.zeros((self.solver.mesh.poly.n_nodes, 2))
        capi.check(capi.lib().fv_adjoint_shape_gradient(self._h, self.solver.mesh.handle, int(objective),
                                                        capi.dptr(r), capi.dptr(out)))
        return out

    def shape_vjp(self, Rbar) -> np.ndarray:
        """(dR/dX)^T Rbar [n_nodes, 2] at the linearisation state."""
        out = np.zeros((self.solver.mesh.poly.n_nodes, 2))
        capi.check(capi.lib().fv_residual_shape_vjp(self._h, self.solver.mesh.handle,
                                                    capi.dptr(np.ascontiguousarray(Rbar, dtype=np.float64)),
                                                    capi.dptr(out)))
        return out

    def freestream_gradient(self, objective: Objective, mach: float, aoa_deg: float, farfield_patches,
                            max_iter: int = 20000, tol: float = 1e-12, method: str = "rk") -> dict:
        """dJ/dM and dJ/dAoA (per degree) of a force coefficient at a
        converged state whose farfield patches carry the freestream
        (1, M cos a, M sin a, 1/gamma) and whose force reference is that
        freestream (q = M^2 / 2, unit chord)."""
        a = np.radians(aoa_deg)
        ref = np.array([1.0, mach * np.cos(a), mach * np.sin(a), 1.0 / self.solver.gas_gamma(), 1.0, 0.25, 0.0])
        self.forward()
        J, g = force_gradient(self.solver, objective, ref)
        lam, fb, hist, it = self.solve(g, max_iter, tol, method)
        fsb = fb[list(farfield_patches)].sum(axis=0)
        dfs_dM = np.array([0.0, np.cos(a), np.sin(a), 0.0])
        dfs_da = np.array([0.0, -mach * np.sin(a), mach * np.cos(a), 0.0])
        # explicit dependence through the force reference (direction, q)
        Jd, _ = force_gradient(self.solver, Objective.Drag, ref)
        Jl, _ = force_gradient(self.solver, Objective.Lift, ref)
        if objective == Objective.Drag:
            eM, ea = -2.0 * J / mach, Jl
        elif objective == Objective.Lift:
            eM, ea = -2.0 * J / mach, -Jd
        else:
            eM, ea = -2.0 * J / mach, 0.0
        dM = eM - fsb @ dfs_dM
        da = (ea - fsb @ dfs_da) * np.pi / 180.0
        r = self.last_residual
        return {"J": J, "dJ_dM": dM, "dJ_dAoA_deg": da, "iterations": it,
                "adjoint_residual": None if r is None else np.asarray(r).tolist()}

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                capi.lib().fv_adjoint_destroy(self._h)
                self._h = None
        except Exception:
            pass


class UnstructuredFVMSolver:
    """GPU scalar diffusion solver with the reference's constructor and methods
    (include/UnstructuredFVMSolver.h:21-92).

    The reference takes each patch's BoundaryType and value from
    ``mesh.patches``; here ``patches`` maps patch name -> (BoundaryType, value)
    (unlisted patches: Dirichlet 0).
    """

    def __init__(self, input_mesh: Mesh, alpha: float, dt: float, initial_value: float, initial_radius: float,
                 patches: Optional[dict] = None):
        if not isinstance(input_mesh, Mesh):
            input_mesh = Mesh(input_mesh)
        self.mesh = input_mesh
        n = len(input_mesh.patch_names)
        pt = np.zeros(max(n, 1), np.int32)
        pv = np.zeros(max(n, 1), np.float64)
        for name, (kind, value) in (patches or {}).items():
            i = input_mesh.patch_names.index(name)
            pt[i] = int(kind)
            pv[i] = float(value)
        h = C.c_void_p()
        capi.check(capi.lib().fv_diffusion_create(input_mesh.handle, float(alpha), float(dt), float(initial_value),
                                                  float(initial_radius), capi.i32ptr(pt), capi.dptr(pv), C.byref(h)))
        self._h = h
        self.n_cells = input_mesh.n_cells

    def step(self) -> None:
        capi.check(capi.lib().fv_diffusion_step(self._h, 1, None))

    def run(self, total_steps: int, history: bool = False):
        out = np.zeros(max(total_steps, 1))
        done = 0
        while done < total_steps:
            k = min(65536, total_steps - done)
            capi.check(capi.lib().fv_diffusion_step(self._h, k, capi.dptr(out[done:]) if history else None))
            done += k
        return out[:total_steps] if history else None

    def field(self) -> np.ndarray:
        out = np.zeros(self.n_cells)
        capi.check(capi.lib().fv_diffusion_get_field(self._h, capi.dptr(out)))
        return out

    def set_field(self, new_phi) -> None:
        p = np.ascontiguousarray(new_phi, dtype=np.float64)
        if p.shape != (self.n_cells,):
            raise ValueError("set_field expects one value per cell")
        capi.check(capi.lib().fv_diffusion_set_field(self._h, capi.dptr(p)))

    def residual_norm(self) -> float:
        out = np.zeros(1)
        capi.check(capi.lib().fv_diffusion_residual(self._h, capi.dptr(out)))
        return float(out[0])

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                capi.lib().fv_diffusion_destroy(h)
            except Exception:
                pass
            self._h = None


class _BatchMesh:
    """Device mesh of concatenated instance meshes (fv_mesh_create_batch)."""

    def __init__(self, meshes: Sequence[Mesh], reorder: str = "morton"):
        self.parts = list(meshes)
        arr = (C.c_void_p * len(self.parts))(*[m.handle.value for m in self.parts])
        h = C.c_void_p()
        capi.check(capi.lib().fv_mesh_create_batch(len(self.parts), arr, capi.REORDER[reorder], C.byref(h)))
        self._h = h
        self.n_cells = sum(m.n_cells for m in self.parts)
        self.offsets = np.cumsum([0] + [m.n_cells for m in self.parts])

    @property
    def handle(self):
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                capi.lib().fv_mesh_destroy(h)
            except Exception:
                pass
            self._h = None


class BatchSolver:
    """Many independent steady Euler solves advanced together.

    ``meshes``: one Mesh per instance (same patches); ``freestreams``:
    (rho, u, v, p) per instance, used by the farfield patches and as the
    initial state; ``boundary_types``: EulerBoundaryType per patch.  Every
    instance stops (is frozen on the device) once its own L2 density
    residual falls below ``tol``.
    """

    def __init__(self, meshes: Sequence[Mesh], boundary_types: Sequence[EulerBoundaryType], freestreams,
                 gamma: float = 1.4, cfl: float = 1.2, flux_scheme: NumericalFluxScheme = NumericalFluxScheme.HLLC,
                 *, order: int = 2, rk_stages: int = 3, gradient: GradientScheme = GradientScheme.LeastSquares,
                 limiter: Limiter = Limiter.Venkatakrishnan, venkat_k: float = 5.0, fp32_flux: bool = False,
                 tol: float = -1.0):
        self.mesh = _BatchMesh(meshes)
        self.n = len(meshes)
        fs = np.array([from_primitive(*q, gamma) for q in freestreams], dtype=np.float64).reshape(-1)
        bc = (capi.BC * len(boundary_types))()
        for i, t in enumerate(boundary_types):
            bc[i].type = int(t)
        o = capi.default_options()
        o.flux, o.order, o.rk_stages, o.dt_mode = int(flux_scheme), int(order), int(rk_stages), 1
        o.gradient, o.limiter, o.venkat_k = int(gradient), int(limiter), float(venkat_k)
        o.precision = 1 if fp32_flux else 0
        self._opt = o
        h = C.c_void_p()
        capi.check(capi.lib().fv_batch_create(self.mesh.handle, bc, len(boundary_types), capi.dptr(fs), float(gamma),
                                              float(cfl), C.byref(o), C.byref(h)))
        self._h = h
        self.set_tolerance(tol)

    def set_tolerance(self, tol: float) -> None:
        capi.check(capi.lib().fv_batch_set_tolerance(self._h, float(tol)))

    @property
    def n_instances(self) -> int:
        return self.n

    # Newton-Krylov over the whole batch (one block-diagonal system, every
    # instance with its own CFL number and stopping test) and limiter
    # freezing for every instance: the single-solver methods apply as is.
    newton = EulerFVMSolver.newton
    freeze_limiter = EulerFVMSolver.freeze_limiter

    def set_field(self, new_U) -> None:
        """Every instance's state [total cells, 4] (the instances' cells one
        after another); the instances' step counters restart."""
        u = np.ascontiguousarray(new_U, dtype=np.float64)
        if u.shape != (self.mesh.n_cells, 4):
            raise ValueError(f"set_field expects shape {(self.mesh.n_cells, 4)}, got {u.shape}")
        capi.check(capi.lib().fv_set_field(self._h, capi.dptr(u)))

    def set_limiter_values(self, psi) -> None:
        """Freeze every instance's limiter at the given values [total cells,
        4] (the instances' cells one after another)."""
        capi.check(capi.lib().fv_solver_limiter_values(self._h, None,
                                                       capi.dptr(np.ascontiguousarray(psi, dtype=np.float64))))

    def limiter_values(self, instance: int) -> np.ndarray:
        """The frozen limiter values [n_cells of the instance, 4]."""
        out = np.zeros((self.mesh.n_cells, 4))
        capi.check(capi.lib().fv_solver_limiter_values(self._h, capi.dptr(out), None))
        o = self.mesh.offsets
        return out[o[instance]:o[instance + 1]]

    def multigrid(self, levels: int = 4, smooth: int = 1, relax: float = 0.7) -> None:
        """Agglomeration multigrid for every instance (agglomerates never
        cross instances; frozen instances get no corrections)."""
        capi.check(capi.lib().fv_solver_multigrid(self._h, self.mesh.handle, int(levels), int(smooth), float(relax)))

    def autotune(self, steps: int = 5, cache: bool = True) -> dict:
        """Launch shapes of the batched kernels chosen by timing (state preserved)."""
        return _autotune(self._h, _shape_key(self._opt, self.mesh.n_cells, True), steps, cache)

    def run(self, n: int) -> None:
        capi.check(capi.lib().fv_step(self._h, int(n), None))

    def step_timed(self, n: int):
        ms = np.zeros(3)
        cnt = np.zeros(3, np.int32)
        capi.check(capi.lib().fv_step_timed(self._h, int(n), capi.dptr(ms), capi.i32ptr(cnt)))
        return ms, cnt

    def set_active(self, instance: int, active: bool) -> None:
        """Freeze or resume one instance (caller-side convergence tests)."""
        capi.check(capi.lib().fv_batch_set_active(self._h, int(instance), int(bool(active))))

    def status(self):
        """(active[n], iterations[n], norms[n, 4])."""
        act = np.zeros(self.n, np.int32)
        it = np.zeros(self.n, np.int32)
        nr = np.zeros((self.n, 4))
        capi.check(capi.lib().fv_batch_status(self._h, capi.i32ptr(act), capi.i32ptr(it), capi.dptr(nr)))
        return act.astype(bool), it, nr

    def field(self, instance: int) -> np.ndarray:
        o = self.mesh.offsets
        return self.field_all()[o[instance]:o[instance + 1]]

    def field_all(self) -> np.ndarray:
        """Every instance's state [total cells, 4], instances one after another."""
        out = np.zeros((self.mesh.n_cells, 4))
        capi.check(capi.lib().fv_get_field(self._h, capi.dptr(out)))
        return out

    def wall_forces(self, instance: int, rho_ref, u_ref, v_ref, p_ref, length_ref=1.0, moment_x=0.25,
                    moment_y=0.0) -> dict:
        ref = np.array([rho_ref, u_ref, v_ref, p_ref, length_ref, moment_x, moment_y], dtype=np.float64)
        out = np.zeros(11)
        capi.check(capi.lib().fv_batch_wall_forces(self._h, int(instance), capi.dptr(ref), capi.dptr(out)))
        keys = ["friction_drag", "pressure_drag", "total_drag", "lift", "moment", "cd_friction", "cd_pressure",
                "cd_total", "cl", "cm", "n_wall_faces"]
        return dict(zip(keys, out.tolist()))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                capi.lib().fv_solver_destroy(h)
            except Exception:
                pass
            self._h = None


class NSBoundaryType(enum.IntEnum):
    """include/NavierStokesFVMSolver.h:19-23 (same numbering)."""
    NoSlipWall = 0
    Farfield = 1
    Outflow = 2


@dataclasses.dataclass
class NSBoundaryCondition:
    """include/NavierStokesFVMSolver.h:25-32."""
    type: NSBoundaryType = NSBoundaryType.NoSlipWall
    wall_u: float = 0.0
    wall_v: float = 0.0
    is_isothermal_wall: bool = False
    wall_temperature: float = 0.0
    farfield_state: Sequence[float] = (0.0, 0.0, 0.0, 0.0)


_NS_TO_ABI = {NSBoundaryType.NoSlipWall: 4, NSBoundaryType.Farfield: 1, NSBoundaryType.Outflow: 2}


class NavierStokesFVMSolver(EulerFVMSolver):
    """GPU Navier-Stokes solver with the reference's constructor and methods
    (include/NavierStokesFVMSolver.h:118-218): the reference's first-order
    scheme with the Jasak-corrected viscous flux.  ``strict`` selects the
    kernels built without FMA contraction in the reference's evaluation
    order; the default build contracts multiply-adds."""

    def __init__(self, input_mesh: Mesh, boundary_conditions: Sequence[NSBoundaryCondition], gamma: float,
                 gas_constant: float, mu: float, prandtl: float, cfl: float,
                 initial_condition: EulerInitialCondition,
                 flux_scheme: NumericalFluxScheme = NumericalFluxScheme.Rusanov,
                 gradient_scheme: GradientScheme = GradientScheme.LeastSquares, exact_riemann_tol: float = 1e-6,
                 exact_riemann_max_iter: int = 20, strict: bool = False):
        arr = (capi.BC * max(1, len(boundary_conditions)))()
        for i, b in enumerate(boundary_conditions):
            arr[i].type = _NS_TO_ABI[NSBoundaryType(b.type)]
            arr[i].isothermal = 1 if b.is_isothermal_wall else 0
            arr[i].wall_u, arr[i].wall_v, arr[i].wall_T = float(b.wall_u), float(b.wall_v), float(b.wall_temperature)
            for k in range(4):
                arr[i].state[k] = float(b.farfield_state[k])
        super().__init__(input_mesh, arr, gamma, cfl, initial_condition, flux_scheme, exact_riemann_tol,
                         exact_riemann_max_iter, gradient=gradient_scheme, strict=strict,
                         _viscous=(gas_constant, mu, prandtl))


@dataclasses.dataclass
class SAModelConstants:
    """SA-noft2 model constants (include/SpalartAllmaras.h:13-23)."""
    cb1: float = 0.1355
    cb2: float = 0.622
    sigma: float = 2.0 / 3.0
    kappa: float = 0.41
    cw2: float = 0.3
    cw3: float = 2.0
    cv1: float = 7.1
    cv2: float = 0.7
    cv3: float = 0.9

    def as_list(self):
        return [self.cb1, self.cb2, self.sigma, self.kappa, self.cw2, self.cw3, self.cv1, self.cv2, self.cv3]


@dataclasses.dataclass
class RANSBoundaryConditionSA:
    """include/RANSTurbulenceSASolver.h: the mean-flow condition plus the
    freestream nu-tilde of a farfield patch."""
    ns: NSBoundaryCondition = dataclasses.field(default_factory=NSBoundaryCondition)
    farfield_nut: float = 0.0


class RANSTurbulenceSASolver(EulerFVMSolver):
    """GPU RANS solver with the Spalart-Allmaras model and the reference's
    constructor and methods (include/RANSTurbulenceSASolver.h): the
    Navier-Stokes scheme with mu + rho nu_t, plus the transported nu-tilde."""

    def __init__(self, input_mesh: Mesh, boundary_conditions: Sequence[RANSBoundaryConditionSA], gamma: float,
                 gas_constant: float, mu: float, prandtl: float, prandtl_t: float, cfl: float,
                 initial_condition: EulerInitialCondition, initial_nut: float,
                 flux_scheme: NumericalFluxScheme = NumericalFluxScheme.Rusanov,
                 gradient_scheme: GradientScheme = GradientScheme.LeastSquares, exact_riemann_tol: float = 1e-6,
                 exact_riemann_max_iter: int = 20, sa_constants: SAModelConstants = None, strict: bool = False):
        arr = (capi.BC * max(1, len(boundary_conditions)))()
        for i, rb in enumerate(boundary_conditions):
            b = rb.ns
            arr[i].type = _NS_TO_ABI[NSBoundaryType(b.type)]
            arr[i].isothermal = 1 if b.is_isothermal_wall else 0
            arr[i].wall_u, arr[i].wall_v, arr[i].wall_T = float(b.wall_u), float(b.wall_v), float(b.wall_temperature)
            for k in range(4):
                arr[i].state[k] = float(b.farfield_state[k])
            arr[i].nut = float(rb.farfield_nut)
        sa = (sa_constants or SAModelConstants()).as_list()
        super().__init__(input_mesh, arr, gamma, cfl, initial_condition, flux_scheme, exact_riemann_tol,
                         exact_riemann_max_iter, gradient=gradient_scheme, strict=strict,
                         _viscous=(gas_constant, mu, prandtl),
                         _rans={"prandtl_t": prandtl_t, "initial_nut": initial_nut, "sa": sa})

    def nut_field(self) -> np.ndarray:
        out = np.zeros(self.n_cells)
        capi.check(capi.lib().fv_get_nut(self._h, capi.dptr(out)))
        return out

    def set_field(self, new_U: np.ndarray, new_nut: np.ndarray = None) -> None:
        super().set_field(new_U)
        if new_nut is not None:
            capi.check(capi.lib().fv_set_nut(self._h, capi.dptr(np.ascontiguousarray(new_nut, dtype=np.float64))))

    def nut_residual(self) -> float:
        r = C.c_double()
        capi.check(capi.lib().fv_get_nut_residual(self._h, C.byref(r)))
        return r.value

    def wall_distance(self) -> np.ndarray:
        out = np.zeros(self.n_cells)
        capi.check(capi.lib().fv_get_wall_distance(self._h, capi.dptr(out)))
        return out


class GradientCalculator:
    """GPU GradientCalculator (include/GradientReconstruction.h:46-83)."""

    def __init__(self, mesh: Mesh, scheme: GradientScheme = GradientScheme.LeastSquares):
        if not isinstance(mesh, Mesh):
            mesh = Mesh(mesh)
        self.mesh = mesh
        h = C.c_void_p()
        capi.check(capi.lib().fv_gradient_create(mesh.handle, int(scheme), C.byref(h)))
        self._h = h

    def compute(self, phi, boundary_phi, face_gradients: bool = False):
        """Cell gradients [N, 2]; with face_gradients also [F, 4] =
        (corrected dphi/dn, corrected gradient x, y, face_normal_distance)."""
        p = np.ascontiguousarray(phi, dtype=np.float64)
        b = np.ascontiguousarray(boundary_phi, dtype=np.float64)
        if p.shape != (self.mesh.n_cells,) or b.shape != (self.mesh.n_faces,):
            raise ValueError("phi must have one value per cell and boundary_phi one per face")
        g = np.zeros((self.mesh.n_cells, 2))
        fo = np.zeros((self.mesh.n_faces, 4)) if face_gradients else None
        capi.check(capi.lib().fv_gradient_compute(self._h, capi.dptr(p), capi.dptr(b), capi.dptr(g),
                                                  capi.dptr(fo) if face_gradients else None))
        return (g, fo) if face_gradients else g

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                capi.lib().fv_gradient_destroy(h)
            except Exception:
                pass
            self._h = None
