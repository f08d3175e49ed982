"""Limiter freezing (fv_solver_freeze_limiter, fv_solver_limiter_values).

No reference counterpart (the reference is first order).  Checks: the
first step after freezing is the unfrozen step bit for bit; frozen values
move between solvers exactly; a transonic solve that limit-cycles through
the limiter converges once the limiter is frozen, and the frozen-limiter
adjoint is then the exact linearisation of the scheme being solved: its
gradients with respect to Mach number and wall-node displacements match
central differences of converged frozen-limiter solves.
"""
import numpy as np
import pytest

from finitevolume_gb300 import meshgen, solvers as S
from helpers import GAMMA

pytestmark = pytest.mark.gpu


def _fs(M, aoa):
    a = np.radians(aoa)
    return np.array([1.0, M * np.cos(a), M * np.sin(a), 1.0 / GAMMA])


def _solver(mesh, fs, rk=3, cfl=1.2, limiter=S.Limiter.Venkatakrishnan):
    bcs = [S.EulerBoundaryCondition(S.EulerBoundaryType.Wall),
           S.EulerBoundaryCondition(S.EulerBoundaryType.CharacteristicFarfield, S.from_primitive(*fs, GAMMA))]
    ic = S.EulerInitialCondition(S.EulerICMode.Freestream, rho=fs[0], u=fs[1], v=fs[2], p=fs[3])
    return S.EulerFVMSolver(mesh, bcs, GAMMA, cfl, ic, S.NumericalFluxScheme.HLLC, order=2, rk_stages=rk,
                            local_dt=True, gradient=S.GradientScheme.LeastSquares, limiter=limiter)


def _converge(s, tol, max_iter, chunk=500):
    done, last = 0, np.inf
    while done < max_iter:
        h = s.run(chunk, history=True)
        done += chunk
        last = float(h[-1, 0])
        if last < tol or not np.isfinite(last):
            break
    return last


def test_first_frozen_step_is_the_unfrozen_step(gpu):
    mesh = S.Mesh(meshgen.naca_ogrid(96, 48))
    fs = _fs(0.75, 2.0)
    a = _solver(mesh, fs, rk=1, cfl=0.5)
    a.run(200)
    U = a.field()
    a.set_field(U)  # both solvers start from primitives formed the same way
    b = _solver(mesh, fs, rk=1, cfl=0.5)
    b.set_field(U)
    b.freeze_limiter()
    a.run(1)
    b.run(1)
    assert np.array_equal(a.field(), b.field())
    psi = b.limiter_values()
    assert psi.min() >= 0.0 and psi.max() <= 1.0 and (psi < 1.0).any()
    # released, the limiter is evaluated again: both solvers agree again
    b.freeze_limiter(False)
    a.run(3)
    b.run(3)
    assert np.array_equal(a.field(), b.field())


def test_limiter_values_move_between_solvers(gpu):
    mesh = S.Mesh(meshgen.naca_ogrid(96, 48))
    fs = _fs(0.75, 2.0)
    a = _solver(mesh, fs)
    a.run(300)
    a.freeze_limiter()
    psi = a.limiter_values()
    b = _solver(mesh, fs)
    b.set_field(a.field())
    b.set_limiter_values(psi)
    assert np.array_equal(b.limiter_values(), psi)
    a.run(50)
    b.run(50)
    assert np.array_equal(a.field(), b.field())
    with pytest.raises(S.capi.FVError):
        b.set_limiter_values(np.full_like(psi, 1.5))


def test_frozen_limiter_adjoint_matches_converged_differences(gpu):
    poly = meshgen.naca_ogrid(96, 48, r_far=10.0)
    mesh = S.Mesh(poly)
    M, aoa = 0.75, 2.0
    fs = _fs(M, aoa)
    ref = np.array([1.0, fs[1], fs[2], fs[3], 1.0, 0.25, 0.0])
    tol = 1e-12
    s = _solver(mesh, fs)
    s.multigrid()
    s.run(2000)
    s.freeze_limiter()
    assert _converge(s, tol, 60000) < 1e-11
    psi, U0 = s.limiter_values(), s.field()
    adj = S.DiscreteAdjoint(s)
    gd = adj.freestream_gradient(S.Objective.Drag, M, aoa, [1], max_iter=200000, tol=1e-13)
    _, g = S.force_gradient(s, S.Objective.Lift, ref)
    adj.solve(g, 200000, 1e-13)
    gl = adj.shape_gradient(S.Objective.Lift, ref)

    def frozen_solve(m, nodes=None):
        sp = _solver(mesh, _fs(m, aoa))
        sp.set_field(U0)
        sp.set_limiter_values(psi)
        if nodes is not None:
            sp.update_nodes(nodes)
        sp.multigrid()
        assert _converge(sp, tol, 60000) < 1e-11
        return sp.wall_forces(1.0, m * np.cos(np.radians(aoa)), m * np.sin(np.radians(aoa)), 1.0 / GAMMA, 1.0,
                              0.25, 0.0)

    hM = 1e-6
    fd = (frozen_solve(M + hM)["cd_total"] - frozen_solve(M - hM)["cd_total"]) / (2 * hM)
    assert abs(gd["dJ_dM"] - fd) <= 1e-4 * abs(fd), (gd["dJ_dM"], fd)
    h = 1e-6
    for d in meshgen.wall_normal_directions(poly, 2, seed=3):
        fd = (frozen_solve(M, poly.nodes + h * d)["cl"] - frozen_solve(M, poly.nodes - h * d)["cl"]) / (2 * h)
        ad = float(np.sum(gl * d))
        assert abs(ad - fd) <= 1e-4 * max(abs(fd), 1e-3), (ad, fd)
