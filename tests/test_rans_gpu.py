"""GPU RANS with the Spalart-Allmaras model (RANSTurbulenceSASolver)
against the reference's outputs.

Fixtures (tests/golden/make_golden.py, the reference compiled in place):
a no-slip NACA0012 O-grid with freestream nu-tilde = 3 nu (Rusanov/HLLC x
LSQ/Green-Gauss) and a channel between an isothermal still wall and a
moving adiabatic wall with outflow ends.  The kernels keep the reference's
evaluation order without FMA contraction; the mean flow, nu-tilde, the
five residual norms and the wall forces agree within 1e-10 relative (the
face geometry goes through std::hypot and the SA destruction through pow,
whose last bits may differ between the fixture's host and this one), and
the wall distance bit for bit.
"""
import numpy as np
import pytest

from finitevolume_gb300 import solvers as S
from helpers import GAMMA, case_of, cons, load_golden, poly_of, rel_err

pytestmark = pytest.mark.gpu

FLUX = {"rusanov": S.NumericalFluxScheme.Rusanov, "hllc": S.NumericalFluxScheme.HLLC}
GRAD = {"lsq": S.GradientScheme.LeastSquares, "gg": S.GradientScheme.GreenGauss}


def _bcs(specs, names):
    out = [S.RANSBoundaryConditionSA()] * len(names)
    for spec in specs:
        p = spec.split(":")
        i = names.index(p[0])
        nut = 0.0
        if p[1] == "noslip":
            b = S.NSBoundaryCondition(S.NSBoundaryType.NoSlipWall)
            if len(p) > 2:
                b.wall_u = float(p[2])
            if len(p) > 3:
                b.wall_v = float(p[3])
            if len(p) > 4:
                b.is_isothermal_wall, b.wall_temperature = True, float(p[4])
        elif p[1] == "outflow":
            b = S.NSBoundaryCondition(S.NSBoundaryType.Outflow)
        else:
            b = S.NSBoundaryCondition(S.NSBoundaryType.Farfield, farfield_state=cons(*map(float, p[2:6])))
            if len(p) > 6:
                nut = float(p[6])
        out[i] = S.RANSBoundaryConditionSA(b, nut)
    return out


def _ic(spec):
    r, u, v, p = map(float, spec.split(":")[1:5])
    return S.EulerInitialCondition(S.EulerICMode.Freestream, rho=r, u=u, v=v, p=p)


def _solver(g, flux, grad, strict=False):
    case = case_of(g)
    poly = poly_of(g)
    return S.RANSTurbulenceSASolver(S.Mesh(poly), _bcs(case["bc"], poly.patch_names), GAMMA, case["R"], case["mu"],
                                    case["Pr"], case["Prt"], case["cfl"], _ic(case["ic"]), case["nut0"], FLUX[flux],
                                    GRAD[grad], strict=strict), case


CASES = [("rans_naca_og64", "rusanov", "lsq"), ("rans_naca_og64", "rusanov", "gg"),
         ("rans_naca_og64", "hllc", "lsq"), ("rans_naca_og64", "hllc", "gg"),
         ("rans_channel_tri", "rusanov", "lsq"), ("rans_channel_tri", "rusanov", "gg")]


@pytest.mark.parametrize("strict", [True, False])
@pytest.mark.parametrize("name,flux,grad", CASES)
def test_rans_sa_vs_reference(gpu, name, flux, grad, strict):
    """Strict (reference evaluation order, no FMA) and default (contracted)
    kernel builds."""
    g = load_golden(name)
    s, case = _solver(g, flux, grad, strict)
    tag = f"{flux}_{grad}"
    assert np.array_equal(s.wall_distance(), g["walld"])
    nut_hist = []
    hist = []
    for _ in range(case["steps"]):
        hist.append(s.run(1, history=True)[-1])
        nut_hist.append(s.nut_residual())
    assert rel_err(s.field(), g[f"field_{tag}"]) < 1e-10
    assert rel_err(s.nut_field(), g[f"nut_{tag}"]) < 1e-10
    ref_hist = g[f"hist_{tag}"]
    np.testing.assert_allclose(np.array(hist), ref_hist[:, :4], rtol=1e-10, atol=1e-300)
    np.testing.assert_allclose(np.array(nut_hist), ref_hist[:, 4], rtol=1e-10)
    f = s.wall_forces(*case["ref"])
    total = g[f"forces_{tag}"][-1]
    keys = ["friction_drag", "pressure_drag", "total_drag", "lift", "moment", "cd_friction", "cd_pressure",
            "cd_total", "cl", "cm"]
    for i, k in enumerate(keys):
        assert abs(f[k] - total[i + 1]) <= 1e-10 * max(1.0, abs(total[i + 1])), k


def test_rans_set_field_keeps_or_replaces_nut(gpu):
    g = load_golden("rans_channel_tri")
    s, case = _solver(g, "rusanov", "lsq")
    s.run(5)
    U, nut = s.field().copy(), s.nut_field().copy()
    s.set_field(U)
    assert np.array_equal(s.nut_field(), nut)
    s.set_field(U, 2.0 * nut)
    assert np.array_equal(s.nut_field(), 2.0 * nut)
