"""The oracle pinned to the reference at the small plain-method configuration's
own size.

tests/golden/config1_og256_ref.npz holds what the reference's own
EulerFVMSolver (compiled in place, tests/golden/make_golden.py) gives on the
NACA0012 O-grid of 256 x 128 quads (32,768 cells), first-order Rusanov,
forward Euler with the global CFL time step at CFL 0.5, slip wall and
fixed-state farfield, M 0.5, AoA 2 deg, after 3,000 iterations: the field,
the 3,000 x 4 residual history and the inviscid wall forces of
compute_wall_forces (src/WallTraction.cpp:163-217).  The fixture carries the
mesh it was made on (meshgen.naca_ogrid(256, 128) on the host that made it).
"""
import numpy as np

from helpers import case_of, load_golden, parse_bcs, parse_ic, poly_of, FLUX_ID, GAMMA
from oracle import port

TOL = 1e-10


def config1_mesh(g):
    poly = poly_of(g)
    assert poly.n_cells == 256 * 128
    return poly


def test_oracle_reproduces_reference_config1_at_full_size():
    g = load_golden("config1_og256_ref")
    case = case_of(g)
    poly = config1_mesh(g)
    assert poly.n_cells == 32768
    om = port.OracleMesh(poly)
    e = port.OracleEuler(om, parse_bcs(case["bc"], poly.patch_names), gamma=GAMMA, cfl=case["cfl"],
                         ic=parse_ic(case["ic"]), flux=FLUX_ID[case["flux"]])
    hist = e.run(case["steps"])
    assert np.array_equal(e.field(), g["field"])
    np.testing.assert_allclose(hist, g["hist"], rtol=TOL, atol=0)
    is_wall = np.array([1 if b.split(":")[1] == "wall" else 0 for b in case["bc"]], np.intc)
    order = [poly.patch_names.index(b.split(":")[0]) for b in case["bc"]]
    wall = np.zeros(len(poly.patch_names), np.intc)
    wall[order] = is_wall
    f = e.wall_forces(wall, np.array(case["ref"]))
    total = g["forces"][g["forces"][:, 0] == -1][0]
    np.testing.assert_allclose(f[:10], total[1:11], rtol=TOL, atol=1e-15)
