"""GPU parity at the configurations' own sizes.

- The small plain-method configuration in the reference's mode (NACA0012
  O-grid 256 x 128 = 32,768 cells, first-order Rusanov, forward Euler,
  global CFL time step, fixed-state farfield, 3,000 iterations) against the
  reference's own output (tests/golden/config1_og256_ref.npz): the strict
  kernels give its field bit for bit, the default (FMA-contracted) kernels
  within 1e-10; residual history and CL/CD within 1e-10.
- The same configuration as specified for this build (local time stepping,
  characteristic farfield), which the reference cannot run: against the
  oracle port (oracle/fv_oracle.cpp, the reference's loop with the two
  extensions), 3,000 iterations, CL, CD, density history and field within
  1e-10.
- The headline workload (2nd-order HLLC, least squares, Venkatakrishnan
  K = 5, SSP-RK3 at CFL 1.2, local dt, M 0.8, AoA 1.25 deg) on the full
  968,907-cell mixed mesh: a few iterations from the benchmark's start state,
  GPU against the oracle port, field within 1e-10.

Reference: src/EulerFVMSolver.cpp:58-162 (step, compute_dt),
src/WallTraction.cpp:163-217 (forces).
"""
import numpy as np
import pytest

from finitevolume_gb300 import meshgen, solvers as S
from helpers import case_of, load_golden, parse_bcs, parse_ic, gpu_solver, rel_err, GAMMA
from oracle import port
from test_config1_oracle import config1_mesh

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _wall_mask(case, poly):
    wall = np.zeros(len(poly.patch_names), np.intc)
    for b in case["bc"]:
        name, kind = b.split(":")[:2]
        wall[poly.patch_names.index(name)] = 1 if kind == "wall" else 0
    return wall


@pytest.mark.parametrize("strict", [True, False])
def test_config1_reference_mode_matches_reference(gpu, strict):
    g = load_golden("config1_og256_ref")
    case = case_of(g)
    poly = config1_mesh(g)
    s = gpu_solver(poly, parse_bcs(case["bc"], poly.patch_names), parse_ic(case["ic"]), case["flux"],
                   cfl=case["cfl"], strict=strict)
    hist = s.run(case["steps"], history=True)
    field = s.field()
    if strict:
        assert np.array_equal(field, g["field"])
    else:
        assert rel_err(field, g["field"]) <= TOL
    np.testing.assert_allclose(hist, g["hist"], rtol=TOL, atol=0)
    f = s.wall_forces(*case["ref"])
    total = g["forces"][g["forces"][:, 0] == -1][0]
    keys = ["friction_drag", "pressure_drag", "total_drag", "lift", "moment", "cd_friction", "cd_pressure",
            "cd_total", "cl", "cm"]
    np.testing.assert_allclose([f[k] for k in keys], total[1:11], rtol=TOL, atol=1e-15)


def test_config1_local_dt_characteristic_farfield_matches_oracle(gpu):
    M, aoa = 0.5, np.radians(2.0)
    r, u, v, p = 1.0, M * np.cos(aoa), M * np.sin(aoa), 1.0 / GAMMA
    st = list(S.from_primitive(r, u, v, p, GAMMA))
    poly = meshgen.naca_ogrid(256, 128)
    steps = 3000
    bcs = [(0, [0.0] * 4), (3, st)]
    ic = {"mode": "free", "rho": r, "u": u, "v": v, "p": p}
    e = port.OracleEuler(port.OracleMesh(poly), bcs, gamma=GAMMA, cfl=0.5, ic=ic, flux=0, local_dt=True)
    ohist = e.run(steps)
    s = gpu_solver(poly, bcs, ic, "rusanov", cfl=0.5, local_dt=True)
    hist = s.run(steps, history=True)
    assert rel_err(s.field(), e.field()) <= TOL
    np.testing.assert_allclose(hist[:, 0], ohist[:, 0], rtol=TOL, atol=0)
    ref = np.array([r, u, v, p, 1.0, 0.25, 0.0])
    of = e.wall_forces(np.array([1, 0], np.intc), ref)
    f = s.wall_forces(*ref)
    assert abs(f["cl"] - of[8]) <= TOL * abs(of[8])
    assert abs(f["cd_total"] - of[7]) <= TOL * abs(of[7])


def test_headline_mixed_1M_matches_oracle_port(gpu):
    import bench
    poly = bench.load_mesh()
    assert 0.95e6 < poly.n_cells < 1.0e6
    iters = 3
    ref = bench.port_solver(poly)  # starts from bench.initial_state
    ref.run(iters)
    s, _ = bench.make_solver(poly)  # likewise
    s.run(iters)
    assert rel_err(s.field(), ref.field()) <= TOL
