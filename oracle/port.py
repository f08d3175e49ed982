"""ORACLE -- test infrastructure only.

ctypes wrapper of ``oracle/fv_oracle.cpp`` (the CPU restatement of the
reference's residual-and-update loop).  Only the tests, ``__graft_entry__.
smoke()`` and ``bench.py``'s CPU-baseline leg use this module, always as the
checker or the timed CPU baseline, never as part of the product path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfvoracle.so")
_lib = None

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_I64 = C.POINTER(C.c_int64)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            import sys
            sys.path.insert(0, os.path.dirname(HERE))
            from finitevolume_gb300 import build
            build.build_oracle()
        L = C.CDLL(LIB_PATH)
        L.orc_mesh_build.restype = C.c_void_p
        L.orc_mesh_build.argtypes = [C.c_int, _D, C.c_int, _I64, _I, C.c_int, _I, _I, C.c_int]
        L.orc_mesh_free.argtypes = [C.c_void_p]
        L.orc_mesh_counts.argtypes = [C.c_void_p, _I64]
        L.orc_euler_create.restype = C.c_void_p
        L.orc_euler_create.argtypes = [C.c_void_p, _I, _D, _D, _I, _D]
        L.orc_euler_free.argtypes = [C.c_void_p]
        L.orc_flux.argtypes = [C.c_int, _D, _D, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, _D]
        L.orc_euler_run.argtypes = [C.c_void_p, C.c_int, _D]
        L.orc_euler_field.argtypes = [C.c_void_p, _D]
        L.orc_euler_set_field.argtypes = [C.c_void_p, _D]
        L.orc_euler_gradients.argtypes = [C.c_void_p, _D, _D]
        L.orc_euler_set_cfl.argtypes = [C.c_void_p, C.c_double]
        L.orc_euler_wall_forces.argtypes = [C.c_void_p, _I, _D, _D]
        L.orc_diff_create.restype = C.c_void_p
        L.orc_diff_create.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, _I, _D]
        L.orc_diff_free.argtypes = [C.c_void_p]
        L.orc_diff_run.argtypes = [C.c_void_p, C.c_int, _D]
        L.orc_diff_field.argtypes = [C.c_void_p, _D]
        L.orc_rans_create.restype = C.c_void_p
        L.orc_rans_create.argtypes = [C.c_void_p, _I, _D, _D, _I, _D, _I, _D]
        L.orc_rans_free.argtypes = [C.c_void_p]
        L.orc_rans_run.argtypes = [C.c_void_p, C.c_int, _D]
        L.orc_rans_get.argtypes = [C.c_void_p, _D, _D, _D]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_D)


def flux(kind: int, UL, UR, nx: float, ny: float, gamma: float = 1.4, tol: float = 1e-6, maxit: int = 20):
    """One numerical flux of the oracle (0 Rusanov, 1 HLLC, 2 exact Riemann,
    3 the physical flux of UL) through the unit normal (nx, ny)."""
    out = np.zeros(4)
    ul = np.ascontiguousarray(UL, dtype=np.float64)
    ur = np.ascontiguousarray(UR, dtype=np.float64)
    lib().orc_flux(int(kind), ul.ctypes.data_as(_D), ur.ctypes.data_as(_D), nx, ny, gamma, tol, int(maxit),
                   out.ctypes.data_as(_D))
    return out


class OracleMesh:
    def __init__(self, poly):
        L = lib()
        self._keep = [np.ascontiguousarray(poly.nodes, np.float64), np.ascontiguousarray(poly.cell_off, np.int64),
                      np.ascontiguousarray(poly.cell_nodes, np.intc), np.ascontiguousarray(poly.bedges, np.intc),
                      np.ascontiguousarray(poly.bpatch, np.intc)]
        xy, off, cn, be, bp = self._keep
        self.h = L.orc_mesh_build(xy.shape[0], xy.ctypes.data_as(_D), poly.n_cells, off.ctypes.data_as(_I64),
                                  cn.ctypes.data_as(_I), be.shape[0], be.ctypes.data_as(_I), bp.ctypes.data_as(_I),
                                  len(poly.patch_names))
        if not self.h:
            raise ValueError("oracle: mesh has untagged boundary faces")
        cnt = np.zeros(2, np.int64)
        L.orc_mesh_counts(self.h, cnt.ctypes.data_as(_I64))
        self.n_cells, self.n_faces = int(cnt[0]), int(cnt[1])
        self.n_patches = len(poly.patch_names)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mesh_free(self.h)
            self.h = None


class OracleEuler:
    """CPU Euler solver; ``bcs`` is a list of (type, conserved_state) per patch.

    ic: dict with mode 'free' (rho,u,v,p) or 'two' (rho_l..p_r, x0).
    """

    def __init__(self, mesh: OracleMesh, bcs, gamma=1.4, cfl=0.5, ic=None, flux=0, tol=1e-6, maxit=20, order=1,
                 rk=1, local_dt=False, gradient=0, limiter=2, venkat_k=5.0):
        ic = ic or {"mode": "free", "rho": 1.0, "u": 0.0, "v": 0.0, "p": 1.0}
        if ic["mode"] == "free":
            icv = [0.0, ic["rho"], ic["u"], ic["v"], ic["p"]] + [0.0] * 9
        else:
            icv = [1.0, 0, 0, 0, 0, ic["rho_l"], ic["u_l"], ic["v_l"], ic["p_l"], ic["rho_r"], ic["u_r"], ic["v_r"],
                   ic["p_r"], ic["x0"]]
        bt = np.array([int(t) for t, _ in bcs], dtype=np.intc)
        bs = np.array([list(s) for _, s in bcs], dtype=np.float64).reshape(-1)
        iopt = np.array([flux, order, rk, 1 if local_dt else 0, gradient, limiter, maxit, 0], dtype=np.intc)
        dopt = np.array([gamma, cfl, tol, venkat_k], dtype=np.float64)
        self.mesh = mesh
        self.n_cells = mesh.n_cells
        self.h = lib().orc_euler_create(mesh.h, bt.ctypes.data_as(_I), _d(bs), _d(np.array(icv)),
                                        iopt.ctypes.data_as(_I), _d(dopt))

    def run(self, n: int) -> np.ndarray:
        hist = np.zeros((n, 4))
        lib().orc_euler_run(self.h, n, hist.ctypes.data_as(_D))
        return hist

    def field(self) -> np.ndarray:
        out = np.zeros((self.n_cells, 4))
        lib().orc_euler_field(self.h, out.ctypes.data_as(_D))
        return out

    def set_field(self, U) -> None:
        u = np.ascontiguousarray(U, np.float64)
        lib().orc_euler_set_field(self.h, u.ctypes.data_as(_D))

    def set_cfl(self, c: float) -> None:
        lib().orc_euler_set_cfl(self.h, c)

    def gradients(self):
        """(limited gradients N x 8 as gx[4], gy[4]; primitives N x 4) of the current state."""
        g = np.zeros((self.n_cells, 8))
        w = np.zeros((self.n_cells, 4))
        lib().orc_euler_gradients(self.h, g.ctypes.data_as(_D), w.ctypes.data_as(_D))
        return g, w

    def wall_forces(self, is_wall, ref):
        out = np.zeros(11)
        w = np.ascontiguousarray(is_wall, np.intc)
        lib().orc_euler_wall_forces(self.h, w.ctypes.data_as(_I), _d(ref), out.ctypes.data_as(_D))
        return out

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_euler_free(self.h)
            self.h = None


class OracleDiffusion:
    def __init__(self, mesh: OracleMesh, alpha, dt, v0, r0, ptype, pval):
        self.n_cells = mesh.n_cells
        pt = np.ascontiguousarray(ptype, np.intc)
        self.h = lib().orc_diff_create(mesh.h, alpha, dt, v0, r0, pt.ctypes.data_as(_I), _d(pval))

    def run(self, n):
        hist = np.zeros(n)
        lib().orc_diff_run(self.h, n, hist.ctypes.data_as(_D))
        return hist

    def field(self):
        out = np.zeros(self.n_cells)
        lib().orc_diff_field(self.h, out.ctypes.data_as(_D))
        return out

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_diff_free(self.h)
            self.h = None


class OracleRANS:
    """CPU RANS-SA solver (RANSTurbulenceSASolver).  ``bcs``: per patch a dict
    with ``type`` ("noslip", "farfield", "outflow"), and as the kind needs
    ``state`` (conserved farfield state), ``nut`` (farfield nu-tilde),
    ``wall_u``, ``wall_v``, ``wall_T`` (isothermal when given).  ``ic`` as
    :class:`OracleEuler`; ``flux`` 0 Rusanov / 1 HLLC / 2 exact, ``gradient``
    0 least squares / 1 Green-Gauss."""

    KINDS = {"noslip": 4, "farfield": 1, "outflow": 2}

    def __init__(self, mesh: OracleMesh, bcs, gamma, R, mu, Pr, Prt, cfl, ic, nut0, flux=0, gradient=0, tol=1e-6,
                 maxit=20):
        icv = [0.0, ic["rho"], ic["u"], ic["v"], ic["p"]] + [0.0] * 9
        bt = np.array([self.KINDS[b["type"]] for b in bcs], dtype=np.intc)
        bs = np.array([list(b.get("state", (0.0, 0.0, 0.0, 0.0))) for b in bcs], dtype=np.float64).reshape(-1)
        bw = np.array([[b.get("wall_u", 0.0), b.get("wall_v", 0.0), b.get("wall_T", 0.0), b.get("nut", 0.0)]
                       for b in bcs], dtype=np.float64).reshape(-1)
        iso = np.array([1 if "wall_T" in b else 0 for b in bcs], dtype=np.intc)
        iopt = np.array([flux, gradient, maxit], dtype=np.intc)
        dopt = np.array([gamma, R, mu, Pr, Prt, cfl, tol, nut0], dtype=np.float64)
        self.mesh = mesh
        self.n_cells = mesh.n_cells
        self.h = lib().orc_rans_create(mesh.h, bt.ctypes.data_as(_I), _d(bs), _d(bw), iso.ctypes.data_as(_I),
                                       _d(np.array(icv)), iopt.ctypes.data_as(_I), _d(dopt))

    def run(self, n: int) -> np.ndarray:
        """n steps; history [n, 5] (rho, rho_u, rho_v, E and nu-tilde residual norms)."""
        hist = np.zeros((n, 5))
        lib().orc_rans_run(self.h, n, hist.ctypes.data_as(_D))
        return hist

    def get(self):
        """(conserved field [N, 4], nu-tilde [N], wall distance [N])."""
        f, nt, wd = np.zeros((self.n_cells, 4)), np.zeros(self.n_cells), np.zeros(self.n_cells)
        lib().orc_rans_get(self.h, f.ctypes.data_as(_D), nt.ctypes.data_as(_D), wd.ctypes.data_as(_D))
        return f, nt, wd

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_rans_free(self.h)
            self.h = None


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def num_threads() -> int:
    return int(lib().orc_num_threads())
