"""Newton-Krylov steady solves (fv_steady_newton).

The reference reaches steady states with its explicit loop only
(EulerFVMSolver::step, src/EulerFVMSolver.cpp:58-112), so the test of the
Newton path is that it drives the same discrete residual to zero:

- a subsonic second-order HLLC case converges below 1e-12 and the state it
  leaves is a fixed point of the explicit scheme (one explicit step from it
  leaves the density residual below 1e-11);
- its CL and CD agree with the explicit solver's run to its own steady
  state (the same discrete solution reached two ways);
- a batch of uneven instances (mesh size, Mach, AoA) solved as one
  block-diagonal system converges per instance, and every instance's field
  equals its standalone Newton solve (1e-8 relative: both are converged to
  1e-12 along different paths, not bit for bit);
- the Krylov adjoint at a Newton-converged transonic state matches central
  differences of Newton solves (1e-4 relative);
- the options are validated before any device work.
"""
import numpy as np
import pytest

from finitevolume_gb300 import capi, meshgen, solvers as S
from helpers import GAMMA, rel_err

pytestmark = pytest.mark.gpu


def _fs(M, aoa):
    a = np.radians(aoa)
    return (1.0, M * np.cos(a), M * np.sin(a), 1.0 / GAMMA)


def _solver(poly, M, aoa):
    fs = _fs(M, aoa)
    bcs = [S.EulerBoundaryCondition(S.EulerBoundaryType.Wall),
           S.EulerBoundaryCondition(S.EulerBoundaryType.CharacteristicFarfield, S.from_primitive(*fs, GAMMA))]
    ic = S.EulerInitialCondition(S.EulerICMode.Freestream, rho=fs[0], u=fs[1], v=fs[2], p=fs[3])
    s = S.EulerFVMSolver(S.Mesh(poly), bcs, GAMMA, 1.2, ic, S.NumericalFluxScheme.HLLC, order=2, rk_stages=3,
                         local_dt=True, gradient=S.GradientScheme.LeastSquares, limiter=S.Limiter.Venkatakrishnan,
                         venkat_k=5.0)
    return s, fs


def test_newton_converges_to_the_explicit_schemes_steady_state(gpu):
    poly = meshgen.naca_ogrid(64, 32)
    s, fs = _solver(poly, 0.5, 2.0)
    s.run(100)
    s.freeze_limiter(True)
    h, it = s.newton(max_newton=120, tol=1e-12)
    assert it < 120 and h[-1, 0] < 1e-12
    assert np.isfinite(h).all()
    ref = (*fs, 1.0, 0.25, 0.0)
    f_newton = s.wall_forces(*ref)
    # a fixed point of the explicit (frozen-limiter) scheme
    s.run(1)
    assert s.residual().as_array()[0] < 1e-11
    # the explicit solver on its own reaches the same discrete solution
    e, _ = _solver(poly, 0.5, 2.0)
    e.run(100)
    e.set_limiter_values(s.limiter_values())
    e.multigrid(levels=4)
    for _ in range(200):
        e.run(500)
        if e.residual().as_array()[0] < 1e-12:
            break
    assert e.residual().as_array()[0] < 1e-12
    f_explicit = e.wall_forces(*ref)
    assert abs(f_newton["cl"] - f_explicit["cl"]) <= 1e-8 * abs(f_explicit["cl"])
    assert abs(f_newton["cd_total"] - f_explicit["cd_total"]) <= 1e-8 + 1e-6 * abs(f_explicit["cd_total"])


def test_batched_newton_instances_match_standalone_newton(gpu):
    cases = [("2412", 48, 24, 0.5, 2.0), ("0012", 64, 32, 0.6, -1.0), ("4415", 40, 20, 0.3, 5.0)]
    polys = [meshgen.naca_ogrid(ni, nj, code=code) for code, ni, nj, _, _ in cases]
    fss = [_fs(M, a) for *_, M, a in cases]
    b = S.BatchSolver([S.Mesh(p) for p in polys],
                      [S.EulerBoundaryType.Wall, S.EulerBoundaryType.CharacteristicFarfield], fss)
    b.run(100)
    b.freeze_limiter(True)
    h, it = b.newton(max_newton=150, tol=1e-12)
    steps = b.last_newton_instance_steps
    assert (steps >= 0).all() and it <= 150
    for i, (p, (_, _, _, M, a)) in enumerate(zip(polys, cases)):
        s, _ = _solver(p, M, a)
        s.run(100)
        s.set_limiter_values(b.limiter_values(i))
        _, k = s.newton(max_newton=150, tol=1e-12)
        assert k < 150
        assert rel_err(b.field(i), s.field()) < 1e-8


def test_newton_rejects_bad_options(gpu):
    poly = meshgen.naca_ogrid(32, 16)
    s, _ = _solver(poly, 0.5, 2.0)
    u0 = s.field().copy()
    for kw in ({"krylov_dim": 0}, {"krylov_dim": 201}, {"cfl0": -1.0}, {"cfl_growth": 0.5}, {"precond_kind": 3},
               {"precond_sweeps": 0}, {"max_rel_change": 0.0}):
        with pytest.raises(capi.FVError):
            s.newton(max_newton=5, **kw)
    assert np.array_equal(s.field(), u0)


def test_krylov_adjoint_matches_differences_of_newton_solves(gpu):
    """The pseudo-transient Krylov adjoint (fv_adjoint_solve_krylov) at a
    Newton-converged transonic state (frozen limiter): dCD/dM and dCD/dAoA
    against central differences of Newton solves converged to 1e-13 from the
    base state with the limiter frozen at the same values."""
    poly = meshgen.naca_ogrid(64, 32)
    M, aoa = 0.75, 2.0
    s, fs = _solver(poly, M, aoa)
    s.run(300)
    s.freeze_limiter(True)
    h, _ = s.newton(max_newton=200, tol=1e-12)
    assert h[-1, 0] < 1e-12
    U0, psi = s.field().copy(), s.limiter_values()
    adj = S.DiscreteAdjoint(s, full_limiter=False)
    gd = adj.freestream_gradient(S.Objective.Drag, M, aoa, [1], max_iter=20000, tol=1e-11, method="krylov")
    assert max(gd["adjoint_residual"]) < 1e-9

    def cd_at(m, al):
        sp, f = _solver(poly, m, al)
        sp.set_limiter_values(psi)
        sp.set_field(U0)
        hh, _ = sp.newton(max_newton=200, tol=1e-13)
        assert hh[-1, 0] < 1e-13
        return sp.wall_forces(*f, 1.0, 0.25, 0.0)["cd_total"]

    hM, ha = 1e-6, 1e-5
    fd_m = (cd_at(M + hM, aoa) - cd_at(M - hM, aoa)) / (2 * hM)
    fd_a = (cd_at(M, aoa + ha) - cd_at(M, aoa - ha)) / (2 * ha)
    assert abs(gd["dJ_dM"] - fd_m) <= 1e-4 * abs(fd_m), (gd["dJ_dM"], fd_m)
    assert abs(gd["dJ_dAoA_deg"] - fd_a) <= 1e-4 * abs(fd_a), (gd["dJ_dAoA_deg"], fd_a)
