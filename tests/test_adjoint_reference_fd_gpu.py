"""The discrete adjoint against differences of the reference solver itself.

tests/golden/adjoint_fd_ref.npz holds drag and lift of the reference's own
EulerFVMSolver (compiled in place, tests/golden/make_golden.py), converged
to its round-off floor (final residual norms ~5e-13) on a NACA0012 O-grid
of 64 x 32 cells with the first-order scheme and the fixed-state farfield
at M 0.5, AoA 2 deg and at M +- 1e-4, AoA +- 1e-3 deg, for the Rusanov and
HLLC fluxes; forces by compute_wall_forces with zero viscosity
(src/WallTraction.cpp:163-217) against the freestream.  The GPU solver
converges the same discrete problem, and its discrete adjoint's dCD/dM,
dCD/dAoA, dCL/dM and dCL/dAoA must match the reference's central
differences within 1e-4 relative.
"""
import numpy as np
import pytest

from finitevolume_gb300 import solvers as S
from helpers import case_of, load_golden, poly_of, GAMMA

pytestmark = pytest.mark.gpu

FLUX = {"rusanov": S.NumericalFluxScheme.Rusanov, "hllc": S.NumericalFluxScheme.HLLC}


def _fs(M, aoa):
    a = np.radians(aoa)
    return np.array([1.0, M * np.cos(a), M * np.sin(a), 1.0 / GAMMA])


@pytest.mark.parametrize("flux", ["rusanov", "hllc"])
def test_adjoint_matches_reference_solver_differences(gpu, flux):
    g = load_golden("adjoint_fd_ref")
    case = case_of(g)
    poly = poly_of(g)
    M, aoa = case["mach"], case["aoa_deg"]
    fs = _fs(M, aoa)
    bcs = [S.EulerBoundaryCondition(S.EulerBoundaryType.Wall),
           S.EulerBoundaryCondition(S.EulerBoundaryType.Farfield, S.from_primitive(*fs, GAMMA))]
    ic = S.EulerInitialCondition(S.EulerICMode.Freestream, rho=fs[0], u=fs[1], v=fs[2], p=fs[3])
    # the reference's scheme (first order, forward Euler), local dt to reach
    # the same steady state sooner
    s = S.EulerFVMSolver(S.Mesh(poly), bcs, GAMMA, 0.9, ic, FLUX[flux], local_dt=True)
    for _ in range(60):
        h = s.run(1000, history=True)
        if h[:, 0].min() < 1e-12:
            break
    assert h[:, 0].min() < 1e-12
    s.run(10000)  # on to the round-off floor, where the reference's runs ended
    P = g[f"points_{flux}"]  # mach, aoa_deg, cd_total, cl
    ref = np.array([1.0, fs[1], fs[2], fs[3], 1.0, 0.25, 0.0])
    f = s.wall_forces(*ref)
    # the same steady state as the reference's (both at their round-off floor)
    assert abs(f["cd_total"] - P[0, 2]) <= 1e-8 * abs(P[0, 2])
    assert abs(f["cl"] - P[0, 3]) <= 1e-8 * abs(P[0, 3])
    hM, ha = case["h_mach"], case["h_aoa_deg"]
    fd = {"cd_M": (P[1, 2] - P[2, 2]) / (2 * hM), "cd_a": (P[3, 2] - P[4, 2]) / (2 * ha),
          "cl_M": (P[1, 3] - P[2, 3]) / (2 * hM), "cl_a": (P[3, 3] - P[4, 3]) / (2 * ha)}
    adj = S.DiscreteAdjoint(s)
    gd = adj.freestream_gradient(S.Objective.Drag, M, aoa, [1], max_iter=60000, tol=1e-12)
    gl = adj.freestream_gradient(S.Objective.Lift, M, aoa, [1], max_iter=60000, tol=1e-12)
    ad = {"cd_M": gd["dJ_dM"], "cd_a": gd["dJ_dAoA_deg"], "cl_M": gl["dJ_dM"], "cl_a": gl["dJ_dAoA_deg"]}
    for k in fd:
        assert abs(ad[k] - fd[k]) <= 1e-4 * max(abs(fd[k]), 1e-3), (k, ad[k], fd[k])
