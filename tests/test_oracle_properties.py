"""Properties of the CPU oracle's second-order scheme (oracle/fv_oracle.cpp).

The reference is first order, so MUSCL reconstruction, the limiters, SSP-RK3
and local time stepping have no reference output to pin them; the GPU
kernels are checked against this CPU definition.  These tests check the
definition itself against properties any consistent finite-volume scheme
has, on the CPU:

- a uniform freestream is preserved exactly when every boundary is a
  farfield at that state (the residual vanishes to round-off);
- with slip walls all round and a global time step, mass and total energy
  are conserved to round-off (face fluxes cancel between neighbours and a
  mirrored wall state carries no mass or energy flux), first and second
  order, forward Euler and SSP-RK3;
- least-squares gradients are exact for a linear field in every interior
  cell, and limiting never raises a gradient's magnitude.
"""
import numpy as np
import pytest

from finitevolume_gb300 import meshgen, solvers as S
from helpers import GAMMA, cons
from oracle import port

RUSANOV, HLLC = 0, 1


def _prim_state(rho, u, v, p):
    return list(cons(rho, u, v, p))


def _geometry(poly):
    ex = S.Mesh(poly).export()
    fi, cd = ex["faces_i32"], ex["cells_f64"]
    boundary_cells = np.unique(fi[fi[:, 3] < 0, 2])
    return cd[:, 0], cd[:, 1], cd[:, 2], boundary_cells


@pytest.mark.parametrize("flux", [RUSANOV, HLLC])
@pytest.mark.parametrize("gradient,limiter", [(0, 2), (0, 1), (1, 2)])
@pytest.mark.parametrize("farfield", [1, 3])
def test_uniform_freestream_is_preserved(flux, gradient, limiter, farfield):
    poly = meshgen.naca_ogrid(32, 16)
    r, u, v, p = 1.0, 0.5 * np.cos(0.1), 0.5 * np.sin(0.1), 1.0 / GAMMA
    st = _prim_state(r, u, v, p)
    e = port.OracleEuler(port.OracleMesh(poly), [(farfield, st), (farfield, st)], gamma=GAMMA, cfl=0.8,
                         ic={"mode": "free", "rho": r, "u": u, "v": v, "p": p}, flux=flux, order=2, rk=3,
                         local_dt=True, gradient=gradient, limiter=limiter)
    U0 = e.field()
    hist = e.run(20)
    scale = np.abs(U0).max(axis=0)
    assert np.abs(e.field() - U0).max(axis=0).max() <= 1e-13 * scale.max()
    assert hist.max() <= 1e-12


@pytest.mark.parametrize("order,rk", [(1, 1), (2, 1), (2, 3)])
@pytest.mark.parametrize("flux", [RUSANOV, HLLC])
def test_closed_box_conserves_mass_and_energy(order, rk, flux):
    poly = meshgen.wavy_quads(16, 0.03)
    vol, cx, cy, _ = _geometry(poly)
    om = port.OracleMesh(poly)
    wall = (0, [0.0] * 4)
    e = port.OracleEuler(om, [wall] * 4, gamma=GAMMA, cfl=0.4, flux=flux, order=order, rk=rk, local_dt=False,
                         gradient=0, limiter=2)
    # a smooth non-uniform start with motion towards every wall
    rho = 1.0 + 0.2 * np.sin(np.pi * cx) * np.sin(np.pi * cy)
    uu = 0.3 * np.cos(np.pi * cy) * (cx - 0.5)
    vv = -0.2 * np.cos(np.pi * cx) * (cy - 0.4)
    pp = 1.0 + 0.3 * np.exp(-20 * ((cx - 0.4) ** 2 + (cy - 0.6) ** 2))
    U = np.stack(cons(rho, uu, vv, pp), 1)
    e.set_field(U)
    m0, E0 = float(np.sum(vol * U[:, 0])), float(np.sum(vol * U[:, 3]))
    hist = e.run(50)
    assert np.isfinite(hist).all()
    U1 = e.field()
    assert np.abs(U1 - U).max() > 1e-3  # the flow did evolve
    assert abs(float(np.sum(vol * U1[:, 0])) - m0) <= 1e-13 * m0
    assert abs(float(np.sum(vol * U1[:, 3])) - E0) <= 1e-13 * E0


def test_least_squares_gradients_exact_for_linear_fields():
    poly = meshgen.naca_ogrid(48, 24)
    vol, cx, cy, bcells = _geometry(poly)
    interior = np.setdiff1d(np.arange(vol.size), bcells)
    slopes = np.array([[0.01, -0.02], [0.003, 0.001], [-0.002, 0.004], [0.02, 0.01]])
    base = np.array([1.0, 0.3, 0.1, 1.0 / GAMMA])
    W = base + cx[:, None] * slopes[:, 0] + cy[:, None] * slopes[:, 1]
    U = np.stack(cons(W[:, 0], W[:, 1], W[:, 2], W[:, 3]), 1)
    st = _prim_state(*base)
    results = {}
    for limiter in (0, 2):
        e = port.OracleEuler(port.OracleMesh(poly), [(0, [0.0] * 4), (1, st)], gamma=GAMMA, cfl=0.5, flux=HLLC,
                             order=2, rk=3, local_dt=True, gradient=0, limiter=limiter)
        e.set_field(U)
        g, w = e.gradients()
        np.testing.assert_allclose(w, W, rtol=1e-13, atol=1e-15)
        results[limiter] = g
    g = results[0]
    for k in range(4):
        sc = np.abs(slopes[k]).max()
        np.testing.assert_allclose(g[interior, k], slopes[k, 0], rtol=0, atol=1e-9 * sc)
        np.testing.assert_allclose(g[interior, 4 + k], slopes[k, 1], rtol=0, atol=1e-9 * sc)
    # limiting scales each variable's gradient by psi in [0, 1]
    gl = results[2]
    assert (np.abs(gl) <= np.abs(g) * (1 + 1e-15) + 1e-300).all()
