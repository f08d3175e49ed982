"""Shared helpers for the tests: golden fixtures and case set-up."""
import json
import os

import numpy as np

from finitevolume_gb300.fvmesh import PolyMesh

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GAMMA = 1.4
FLUX_ID = {"rusanov": 0, "hllc": 1, "exact": 2}
BC_ID = {"wall": 0, "farfield": 1, "outflow": 2, "char": 3}


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


def poly_of(g) -> PolyMesh:
    return PolyMesh(g["nodes"], g["cell_off"], g["cell_nodes"], g["bedges"], g["bpatch"],
                    [str(x) for x in g["patch_names"]])


def case_of(g):
    return json.loads(str(g["case"]))


def cons(rho, u, v, p, gamma=GAMMA):
    return [rho, rho * u, rho * v, p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)]


def parse_bcs(spec_list, patch_names, gamma=GAMMA):
    """'name:kind[:rho:u:v:p]' -> list of (type_id, conserved_state) by patch index."""
    out = [(0, [0.0] * 4)] * len(patch_names)
    for spec in spec_list:
        p = spec.split(":")
        idx = patch_names.index(p[0])
        st = cons(*map(float, p[2:6]), gamma) if len(p) >= 6 else [0.0] * 4
        out[idx] = (BC_ID[p[1]], st)
    return out


def parse_ic(spec):
    p = spec.split(":")
    if p[0] == "free":
        return {"mode": "free", "rho": float(p[1]), "u": float(p[2]), "v": float(p[3]), "p": float(p[4])}
    v = list(map(float, p[1:]))
    return {"mode": "two", "rho_l": v[0], "u_l": v[1], "v_l": v[2], "p_l": v[3], "rho_r": v[4], "u_r": v[5],
            "v_r": v[6], "p_r": v[7], "x0": v[8]}


def gpu_solver(mesh, bcs, ic, flux, cfl=0.5, reorder="morton", **kw):
    from finitevolume_gb300 import solvers as S
    m = mesh if isinstance(mesh, S.Mesh) else S.Mesh(mesh, reorder=reorder)
    ebcs = [S.EulerBoundaryCondition(S.EulerBoundaryType(t), st) for t, st in bcs]
    if ic["mode"] == "free":
        eic = S.EulerInitialCondition(S.EulerICMode.Freestream, rho=ic["rho"], u=ic["u"], v=ic["v"], p=ic["p"])
    else:
        eic = S.EulerInitialCondition(S.EulerICMode.TwoRegion, **{k: v for k, v in ic.items() if k != "mode"})
    return S.EulerFVMSolver(m, ebcs, GAMMA, cfl, eic, S.NumericalFluxScheme(FLUX_ID[flux]), **kw)


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
