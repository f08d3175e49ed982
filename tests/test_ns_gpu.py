"""GPU Navier-Stokes (NavierStokesFVMSolver) against the reference's outputs.

The fixtures hold the reference's fields, residual histories and wall
forces for a no-slip NACA0012 O-grid and a channel with an isothermal
moving wall, for Rusanov/HLLC fluxes and LSQ/Green-Gauss viscous gradients.
Both builds of the NS kernels are checked: the strict one (the reference's
evaluation order without FMA contraction) and the default FMA-contracted
one; fields, norms and forces agree within 1e-10 relative.
"""
import numpy as np
import pytest

from finitevolume_gb300 import solvers as S
from helpers import GAMMA, case_of, cons, load_golden, poly_of, rel_err

pytestmark = pytest.mark.gpu

FLUX = {"rusanov": S.NumericalFluxScheme.Rusanov, "hllc": S.NumericalFluxScheme.HLLC}
GRAD = {"lsq": S.GradientScheme.LeastSquares, "gg": S.GradientScheme.GreenGauss}


def _bcs(specs, names):
    out = [S.NSBoundaryCondition()] * len(names)
    for spec in specs:
        p = spec.split(":")
        i = names.index(p[0])
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
        out[i] = b
    return out


def _ic(spec):
    r, u, v, p = map(float, spec.split(":")[1:5])
    return S.EulerInitialCondition(S.EulerICMode.Freestream, rho=r, u=u, v=v, p=p)


CASES = [("ns_naca_og64", "rusanov", "lsq"), ("ns_naca_og64", "rusanov", "gg"), ("ns_naca_og64", "hllc", "lsq"),
         ("ns_naca_og64", "hllc", "gg"), ("ns_channel_tri", "rusanov", "lsq"), ("ns_channel_tri", "rusanov", "gg")]


@pytest.mark.parametrize("strict", [True, False])
@pytest.mark.parametrize("name,flux,grad", CASES)
def test_ns_vs_reference(gpu, name, flux, grad, strict):
    g = load_golden(name)
    case = case_of(g)
    poly = poly_of(g)
    tag = f"{flux}_{grad}"
    s = S.NavierStokesFVMSolver(S.Mesh(poly), _bcs(case["bc"], poly.patch_names), GAMMA, case["R"], case["mu"],
                                case["Pr"], case["cfl"], _ic(case["ic"]), FLUX[flux], GRAD[grad], strict=strict)
    hist = s.run(case["steps"], history=True)
    U = s.field()
    # Within 1e-10 relative: the face geometry of the viscous flux goes through
    # std::hypot, whose last bit may differ between the fixture's host and this one.
    assert rel_err(U, g[f"field_{tag}"]) < 1e-10
    np.testing.assert_allclose(hist, g[f"hist_{tag}"], rtol=1e-10)
    f = s.wall_forces(*case["ref"])
    total = g[f"forces_{tag}"][-1]
    keys = ["friction_drag", "pressure_drag", "total_drag", "lift", "moment", "cd_friction", "cd_pressure",
            "cd_total", "cl", "cm"]
    for i, k in enumerate(keys):
        assert abs(f[k] - total[i + 1]) <= 1e-10 * max(1.0, abs(total[i + 1])), k


def test_overlapping_cells_are_refused(gpu):
    """Two triangles on the same side of their shared edge (both valid
    polygons, positive areas) put the neighbour's centroid behind the face:
    the face-normal distance the viscous time step divides by is negative,
    so the viscous solver refuses the mesh instead of stepping with it."""
    from finitevolume_gb300 import capi
    from finitevolume_gb300.fvmesh import from_cells
    # the second triangle lies below the shared diagonal too, with its
    # centroid further from it than the first one's
    nodes = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [1.5, -0.5]])
    cells = [[0, 1, 2], [0, 3, 2]]
    bedges = np.array([[0, 1], [1, 2], [0, 3], [3, 2]])
    poly = from_cells(nodes, cells, bedges, np.zeros(4, np.int32), ["wall"])
    bcs = [S.NSBoundaryCondition(S.NSBoundaryType.NoSlipWall)]
    ic = S.EulerInitialCondition(S.EulerICMode.Freestream, rho=1.0, u=0.0, v=0.0, p=1.0 / GAMMA)
    with pytest.raises(capi.FVError):
        S.NavierStokesFVMSolver(S.Mesh(poly), bcs, GAMMA, 287.0, 1e-3, 0.72, 0.5, ic,
                                S.NumericalFluxScheme.Rusanov, S.GradientScheme.GreenGauss)
