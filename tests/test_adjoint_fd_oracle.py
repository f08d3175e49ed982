"""The reference-solver difference fixture (tests/golden/adjoint_fd_ref.npz)
pinned by the oracle: the CPU restatement, run as the reference was
(first order, forward Euler, global dt at CFL 0.9, fixed farfield, 80,000
iterations), reproduces the reference's converged base-point field bit for
bit and its drag and lift."""
import numpy as np
import pytest

from helpers import case_of, load_golden, poly_of, cons, FLUX_ID, GAMMA
from oracle import port


@pytest.mark.parametrize("flux", ["rusanov", "hllc"])
def test_oracle_reproduces_reference_converged_base_point(flux):
    g = load_golden("adjoint_fd_ref")
    case = case_of(g)
    poly = poly_of(g)
    M, a = case["mach"], np.radians(case["aoa_deg"])
    r, u, v, p = 1.0, M * np.cos(a), M * np.sin(a), 1.0 / GAMMA
    e = port.OracleEuler(port.OracleMesh(poly), [(0, [0.0] * 4), (1, cons(r, u, v, p))], gamma=GAMMA,
                         cfl=case["cfl"], ic={"mode": "free", "rho": r, "u": u, "v": v, "p": p}, flux=FLUX_ID[flux])
    e.run(case["steps"])
    assert np.array_equal(e.field(), g[f"field_{flux}"])
    f = e.wall_forces(np.array([1, 0], np.intc), np.array([r, u, v, p, 1.0, 0.25, 0.0]))
    P = g[f"points_{flux}"]
    np.testing.assert_allclose([f[7], f[8]], P[0, 2:4], rtol=1e-12)
    assert g[f"final_resid_{flux}"].max() < 1e-12
