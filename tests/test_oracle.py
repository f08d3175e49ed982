"""The CPU oracle is pinned to the reference's own outputs (tests/golden/).

The fixtures were produced by the reference's solver classes compiled in
place (tests/golden/make_golden.py); the oracle restatement must reproduce
their fields bit for bit and their residual histories to the last few ulps
(the L2 sums are OpenMP reductions whose order depends on the thread count).
"""
import numpy as np
import pytest

from helpers import case_of, load_golden, parse_bcs, parse_ic, poly_of, FLUX_ID, GAMMA
from oracle import port


@pytest.mark.parametrize("name", ["naca_og64", "sod_tri"])
@pytest.mark.parametrize("flux", ["rusanov", "hllc", "exact"])
def test_oracle_matches_reference_euler(name, flux):
    g = load_golden(name)
    case = case_of(g)
    poly = poly_of(g)
    om = port.OracleMesh(poly)
    e = port.OracleEuler(om, parse_bcs(case["bc"], poly.patch_names), gamma=GAMMA, cfl=case["cfl"],
                         ic=parse_ic(case["ic"]), flux=FLUX_ID[flux])
    hist = e.run(case["steps"])
    assert np.array_equal(e.field(), g[f"field_{flux}"])
    np.testing.assert_allclose(hist, g[f"hist_{flux}"], rtol=1e-12, atol=0)


def test_oracle_matches_reference_diffusion():
    g = load_golden("diffusion_cart")
    case = case_of(g)
    poly = poly_of(g)
    om = port.OracleMesh(poly)
    pt = np.zeros(len(poly.patch_names), np.intc)
    pv = np.zeros(len(poly.patch_names))
    for spec in case["bc"]:
        n, kind, val = spec.split(":")
        i = poly.patch_names.index(n)
        pt[i] = 1 if kind == "neumann" else 0
        pv[i] = float(val)
    d = port.OracleDiffusion(om, case["alpha"], case["dt"], case["v0"], case["r0"], pt, pv)
    hist = d.run(case["steps"])
    assert np.array_equal(d.field(), g["field"])
    np.testing.assert_allclose(hist, g["hist"], rtol=1e-12)


def test_sod_golden_star_state_plausible():
    """Sanity of the fixture itself: Sod density stays within [0.125, 1]."""
    g = load_golden("sod_tri")
    rho = g["field_exact"][:, 0]
    assert rho.min() > 0.12 and rho.max() < 1.0 + 1e-12
