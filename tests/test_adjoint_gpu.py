"""Discrete adjoint of the Euler residual (fv_residual_forward / _jvp /
_backward / fv_adjoint_solve).

No reference counterpart exists; the checks are the ones an adjoint must
pass against its own primal:
  * transposition: <Rbar, J dU + Jf dfs> == <J^T Rbar, dU> + <Jf^T Rbar, dfs>
    to round-off, for first/second order, Rusanov/HLLC, fixed and
    characteristic farfields (limiter values frozen);
  * linearisation: the tangent map against central differences of the
    residual itself (no limiter, so that freezing it changes nothing);
  * the gradients of drag and lift with respect to Mach number and angle
    of attack from one adjoint solve against central differences of
    converged primal solves.
"""
import numpy as np
import pytest

from finitevolume_gb300 import meshgen, solvers as S
from helpers import GAMMA

pytestmark = pytest.mark.gpu


def _fs(M, aoa):
    a = np.radians(aoa)
    return np.array([1.0, M * np.cos(a), M * np.sin(a), 1.0 / GAMMA])


def _solver(mesh, fs, order, flux, limiter, farfield=S.EulerBoundaryType.CharacteristicFarfield, cfl=1.2):
    bcs = [S.EulerBoundaryCondition(S.EulerBoundaryType.Wall),
           S.EulerBoundaryCondition(farfield, S.from_primitive(*fs, GAMMA))]
    ic = S.EulerInitialCondition(S.EulerICMode.Freestream, rho=fs[0], u=fs[1], v=fs[2], p=fs[3])
    return S.EulerFVMSolver(mesh, bcs, GAMMA, cfl, ic, flux, order=order, rk_stages=3, local_dt=True,
                            gradient=S.GradientScheme.LeastSquares, limiter=limiter)


def _converge(s, tol, max_iter):
    done = 0
    while done < max_iter:
        h = s.run(1000, history=True)
        done += 1000
        if h[:, 0].min() < tol:
            return h[-1, 0]
    return h[-1, 0]


# (order, flux, limiter, farfield kind, Mach): transonic cases are limited
CASES = [(1, S.NumericalFluxScheme.Rusanov, S.Limiter.NoLimiter, S.EulerBoundaryType.CharacteristicFarfield, 0.7),
         (1, S.NumericalFluxScheme.HLLC, S.Limiter.NoLimiter, S.EulerBoundaryType.Farfield, 0.7),
         (2, S.NumericalFluxScheme.HLLC, S.Limiter.Venkatakrishnan, S.EulerBoundaryType.CharacteristicFarfield, 0.7),
         (2, S.NumericalFluxScheme.Rusanov, S.Limiter.BarthJespersen, S.EulerBoundaryType.Farfield, 0.7),
         (2, S.NumericalFluxScheme.HLLC, S.Limiter.NoLimiter, S.EulerBoundaryType.CharacteristicFarfield, 0.5)]


def _mesh(order, **kw):
    # unlimited second order needs the finer grid to stay stable at the nose
    return S.Mesh(meshgen.naca_ogrid(48, 24, **kw) if order == 1 else meshgen.naca_ogrid(96, 48, **kw))


@pytest.mark.parametrize("full", [False, True])
@pytest.mark.parametrize("order,flux,limiter,farfield,mach", CASES)
def test_backward_is_the_transpose_of_forward(gpu, order, flux, limiter, farfield, mach, full):
    mesh = _mesh(order)
    s = _solver(mesh, _fs(mach, 2.0), order, flux, limiter, farfield)
    s.run(300)
    adj = S.DiscreteAdjoint(s, full_limiter=full)
    R = adj.forward()
    assert np.isfinite(R).all()
    rng = np.random.default_rng(7)
    U = s.field()
    dU = rng.standard_normal(U.shape) * np.abs(U).mean(axis=0)
    dfs = rng.standard_normal((2, 4))
    Rb = rng.standard_normal(U.shape)
    lhs = float(np.sum(Rb * adj.jvp(dU, dfs)))
    Ub, fb = adj.vjp(Rb)
    rhs = float(np.sum(Ub * dU) + np.sum(fb * dfs))
    scale = float(np.sum(np.abs(Rb * adj.jvp(dU, dfs))))
    assert abs(lhs - rhs) <= 1e-12 * scale


@pytest.mark.parametrize("order,flux", [(1, S.NumericalFluxScheme.HLLC), (2, S.NumericalFluxScheme.HLLC),
                                        (2, S.NumericalFluxScheme.Rusanov)])
def test_tangent_matches_central_differences(gpu, order, flux):
    mesh = _mesh(order)
    fs = _fs(0.5, 3.0)
    s = _solver(mesh, fs, order, flux, S.Limiter.NoLimiter)
    s.run(300)
    U = s.field()
    adj = S.DiscreteAdjoint(s)
    rng = np.random.default_rng(3)
    dU = rng.standard_normal(U.shape) * np.abs(U).mean(axis=0)
    h = 1e-6
    fd = (adj.forward(U + h * dU) - adj.forward(U - h * dU)) / (2 * h)
    adj.forward(U)
    jv = adj.jvp(dU)
    # Rusanov's max(|Vn| + c) has kinks a central difference can straddle
    assert np.linalg.norm(jv - fd) <= 1e-5 * np.linalg.norm(jv)
    # freestream direction: residual of solvers built on fs +- h dfs, same state
    dfs = np.array([0.1, 0.3, -0.2, 0.05])
    Rp = S.DiscreteAdjoint(_solver(mesh, fs + h * dfs, order, flux, S.Limiter.NoLimiter)).forward(U)
    Rm = S.DiscreteAdjoint(_solver(mesh, fs - h * dfs, order, flux, S.Limiter.NoLimiter)).forward(U)
    fdf = (Rp - Rm) / (2 * h)
    jf = adj.jvp(np.zeros_like(U), np.stack([np.zeros(4), dfs]))
    assert np.linalg.norm(jf - fdf) <= 1e-6 * np.linalg.norm(jf)


def test_full_limiter_tangent_matches_central_differences(gpu):
    """With the limiter active (transonic flow), the full-limiter tangent
    follows central differences of the residual; the frozen one does not.
    (Venkatakrishnan only: Barth-Jespersen's d1/y has no regularisation, so
    in the nearly uniform far field, where y is orders of magnitude below
    any finite perturbation, a difference quotient does not approximate its
    derivative; its full-limiter maps are covered by the transposition
    test.)"""
    mesh = _mesh(2)
    s = _solver(mesh, _fs(0.75, 2.0), 2, S.NumericalFluxScheme.HLLC, S.Limiter.Venkatakrishnan)
    s.run(400)
    U = s.field()
    rng = np.random.default_rng(5)
    dU = rng.standard_normal(U.shape) * np.abs(U).mean(axis=0)
    h = 1e-7
    full = S.DiscreteAdjoint(s, full_limiter=True)
    fd = (full.forward(U + h * dU) - full.forward(U - h * dU)) / (2 * h)
    full.forward(U)
    frozen = S.DiscreteAdjoint(s)
    frozen.forward(U)
    n = np.linalg.norm(fd)
    e_full = np.linalg.norm(full.jvp(dU) - fd) / n
    e_frozen = np.linalg.norm(frozen.jvp(dU) - fd) / n
    assert e_full < 1e-4 and e_frozen > 10 * e_full, (e_full, e_frozen)


def _coefficients(mesh, M, aoa, order, flux, tol, max_iter):
    s = _solver(mesh, _fs(M, aoa), order, flux, S.Limiter.NoLimiter)
    res = _converge(s, tol, max_iter)
    f = s.wall_forces(1.0, M * np.cos(np.radians(aoa)), M * np.sin(np.radians(aoa)), 1.0 / GAMMA, 1.0, 0.25, 0.0)
    return f["cd_total"], f["cl"], res, s


@pytest.mark.parametrize("order", [1, 2])
def test_freestream_gradients_match_converged_differences(gpu, order):
    mesh = _mesh(order, r_far=10.0)
    M, aoa = 0.5, 2.0
    flux = S.NumericalFluxScheme.HLLC
    tol, max_iter = 1e-12, 60000 if order == 1 else 150000
    cd, cl, res, s = _coefficients(mesh, M, aoa, order, flux, tol, max_iter)
    assert res < 1e-11, res
    adj = S.DiscreteAdjoint(s)
    gd = adj.freestream_gradient(S.Objective.Drag, M, aoa, [1], max_iter=max_iter, tol=1e-12)
    gl = adj.freestream_gradient(S.Objective.Lift, M, aoa, [1], max_iter=max_iter, tol=1e-12)
    assert abs(gd["J"] - cd) < 1e-12 and abs(gl["J"] - cl) < 1e-12
    hM, ha = 1e-4, 1e-3
    cdp, clp, r1, _ = _coefficients(mesh, M + hM, aoa, order, flux, tol, max_iter)
    cdm, clm, r2, _ = _coefficients(mesh, M - hM, aoa, order, flux, tol, max_iter)
    cda, cla, r3, _ = _coefficients(mesh, M, aoa + ha, order, flux, tol, max_iter)
    cdb, clb, r4, _ = _coefficients(mesh, M, aoa - ha, order, flux, tol, max_iter)
    assert max(r1, r2, r3, r4) < 1e-11
    fd = {"cd_M": (cdp - cdm) / (2 * hM), "cl_M": (clp - clm) / (2 * hM),
          "cd_a": (cda - cdb) / (2 * ha), "cl_a": (cla - clb) / (2 * ha)}
    ad = {"cd_M": gd["dJ_dM"], "cl_M": gl["dJ_dM"], "cd_a": gd["dJ_dAoA_deg"], "cl_a": gl["dJ_dAoA_deg"]}
    for k in fd:
        assert abs(ad[k] - fd[k]) <= 1e-4 * max(abs(fd[k]), 1e-3), (k, ad[k], fd[k])


def _wall_normal_directions(poly, n_dirs, seed, width=20):
    return meshgen.wall_normal_directions(poly, n_dirs, seed, width)


def _moved(poly, d):
    import dataclasses
    return dataclasses.replace(poly, nodes=np.ascontiguousarray(poly.nodes + d))


@pytest.mark.parametrize("order", [1, 2])
def test_shape_gradient_matches_converged_differences(gpu, order):
    poly = meshgen.naca_ogrid(48, 24, r_far=10.0) if order == 1 else meshgen.naca_ogrid(96, 48, r_far=10.0)
    M, aoa = 0.5, 2.0
    fs = _fs(M, aoa)
    flux = S.NumericalFluxScheme.HLLC
    tol, max_iter = 1e-12, 60000 if order == 1 else 150000
    ref = np.array([1.0, fs[1], fs[2], fs[3], 1.0, 0.25, 0.0])
    s = _solver(S.Mesh(poly), fs, order, flux, S.Limiter.NoLimiter)
    assert _converge(s, tol, max_iter) < 1e-11
    adj = S.DiscreteAdjoint(s)
    adj.forward()
    grads = {}
    for obj in (S.Objective.Lift, S.Objective.Drag):
        _, g = S.force_gradient(s, obj, ref)
        adj.solve(g, max_iter, 1e-12)
        grads[obj] = adj.shape_gradient(obj, ref)
    h = 1e-6
    for d in _wall_normal_directions(poly, 2, seed=11):
        vals = {}
        for sgn in (1, -1):
            sp = _solver(S.Mesh(_moved(poly, sgn * h * d)), fs, order, flux, S.Limiter.NoLimiter)
            assert _converge(sp, tol, max_iter) < 1e-11
            f = sp.wall_forces(*ref)
            vals[sgn] = (f["cl"], f["cd_total"])
        fd_cl = (vals[1][0] - vals[-1][0]) / (2 * h)
        fd_cd = (vals[1][1] - vals[-1][1]) / (2 * h)
        ad_cl = float(np.sum(grads[S.Objective.Lift] * d))
        ad_cd = float(np.sum(grads[S.Objective.Drag] * d))
        assert abs(ad_cl - fd_cl) <= 1e-4 * max(abs(fd_cl), 1e-3), (ad_cl, fd_cl)
        assert abs(ad_cd - fd_cd) <= 1e-4 * max(abs(fd_cd), 1e-3), (ad_cd, fd_cd)


@pytest.mark.parametrize("limiter,full", [(S.Limiter.NoLimiter, False), (S.Limiter.Venkatakrishnan, True)])
def test_residual_shape_cotangent_matches_central_differences(gpu, limiter, full):
    """(dR/dX)^T Rbar against central differences of the residual under a
    smooth displacement of every node (geometry recomputed on the device),
    transonic flow; with the limiter active the full-limiter map includes
    the limiter's geometric inputs and the frozen one misses them."""
    poly = meshgen.naca_ogrid(96, 48, r_far=10.0)
    mesh = S.Mesh(poly)
    s = _solver(mesh, _fs(0.75, 2.0), 2, S.NumericalFluxScheme.HLLC, limiter)
    s.run(400)
    U = s.field()
    X = poly.nodes.copy()
    x, y = X[:, 0], X[:, 1]
    d = 0.1 * np.stack([np.sin(0.7 * x + 0.3 * y), np.cos(0.5 * x - 0.9 * y)], 1)
    d += _wall_normal_directions(poly, 1, seed=4)[0]
    rng = np.random.default_rng(9)
    Rb = rng.standard_normal(U.shape)
    adj = S.DiscreteAdjoint(s, full_limiter=full)
    h = 1e-7
    s.update_nodes(X + h * d)
    Rp = adj.forward(U)
    s.update_nodes(X - h * d)
    Rm = adj.forward(U)
    s.update_nodes(X)
    adj.forward(U)
    fd = float(np.sum(Rb * (Rp - Rm))) / (2 * h)
    scale = float(np.sum(np.abs(Rb * (Rp - Rm)))) / (2 * h)
    e = abs(float(np.sum(adj.shape_vjp(Rb) * d)) - fd) / scale
    assert e < 1e-6, (e, fd, scale)
    if full:
        frozen = S.DiscreteAdjoint(s)
        frozen.forward(U)
        e_frozen = abs(float(np.sum(frozen.shape_vjp(Rb) * d)) - fd) / scale
        assert e_frozen > 10 * e, (e, e_frozen)


def test_gmres_adjoint_matches_pseudo_time_solution(gpu):
    """Where the pseudo-time iteration converges, GMRES on its fixed point
    reaches the same adjoint."""
    mesh = _mesh(2, r_far=10.0)
    fs = _fs(0.5, 2.0)
    s = _solver(mesh, fs, 2, S.NumericalFluxScheme.HLLC, S.Limiter.NoLimiter)
    assert _converge(s, 1e-12, 150000) < 1e-11
    adj = S.DiscreteAdjoint(s)
    adj.forward()
    _, g = S.force_gradient(s, S.Objective.Drag, np.array([1.0, fs[1], fs[2], fs[3], 1.0, 0.25, 0.0]))
    lam_rk, fb_rk, _, _ = adj.solve(g, 150000, 1e-13)
    lam_gm, fb_gm, hist, mv = adj.solve(g, 20000, 1e-10, method="gmres", restart=60)
    assert hist[-1] <= 1e-10 and mv < 20000, (hist[-1], mv)
    assert np.linalg.norm(lam_gm - lam_rk) <= 1e-7 * np.linalg.norm(lam_rk)
    # fsbar = lambda^T dR/dfs inherits lambda's 1e-7 relative agreement
    # (small components to 1e-7 of the largest)
    assert np.allclose(fb_gm, fb_rk, rtol=1e-7, atol=1e-7 * np.abs(fb_rk).max())



def test_frozen_residual_shape_cotangent_matches_central_differences(gpu):
    """With the limiter frozen in the solver (active limiter, transonic
    flow), the frozen-limiter map (dR/dX)^T Rbar against central
    differences of the frozen-limiter residual under node displacements
    (the map the shape-gradient checks of frozen solves rely on)."""
    poly = meshgen.naca_ogrid(96, 48, r_far=10.0)
    mesh = S.Mesh(poly)
    s = _solver(mesh, _fs(0.75, 2.0), 2, S.NumericalFluxScheme.HLLC, S.Limiter.Venkatakrishnan)
    s.run(400)
    s.freeze_limiter()
    assert (s.limiter_values() < 1.0).any()
    U = s.field()
    X = poly.nodes.copy()
    x, y = X[:, 0], X[:, 1]
    rng = np.random.default_rng(3)
    Rb = rng.standard_normal(U.shape)
    adj = S.DiscreteAdjoint(s, full_limiter=False)
    for d in (0.1 * np.stack([np.sin(0.7 * x + 0.3 * y), np.cos(0.5 * x - 0.9 * y)], 1),
              _wall_normal_directions(poly, 1, seed=4)[0]):
        h = 1e-7
        s.update_nodes(X + h * d)
        Rp = adj.forward(U)
        s.update_nodes(X - h * d)
        Rm = adj.forward(U)
        s.update_nodes(X)
        adj.forward(U)
        fd = float(np.sum(Rb * (Rp - Rm))) / (2 * h)
        scale = float(np.sum(np.abs(Rb * (Rp - Rm)))) / (2 * h)
        e = abs(float(np.sum(adj.shape_vjp(Rb) * d)) - fd) / scale
        assert e < 1e-6, (e, fd, scale)
