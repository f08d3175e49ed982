"""Known-answer checks of the oracle's numerical fluxes (CPU).

The reference keeps no test of its flux functions; its design notes record
the properties they were checked for and the Sod star state
(docs/hllc-and-exact-riemann-plan.md:188-201).  The oracle's Rusanov, HLLC
and exact Riemann fluxes (oracle/fv_oracle.cpp, restating
include/RusanovFlux.h, include/HllcFlux.h, include/ExactRiemannFlux.h) are
checked here for:

- consistency, F(U, U, n) = F_phys(U) . n;
- conservation across a face seen from both sides, F(UL, UR, n) =
  -F(UR, UL, -n);
- rotational invariance, F(Q UL, Q UR, Q n) = Q F(UL, UR, n) with Q a
  rotation of the velocity and the normal;
- the Sod problem (rho, p = 1, 1 | 0.125, 0.1 at rest): the exact solver's
  interface flux is the physical flux of the left star state rho*_L =
  0.42632, u* = 0.92745, p* = 0.30313 (the recorded star values, five
  digits), and HLLC's mass flux lies within 10% of it.
"""
import numpy as np
import pytest

from oracle import port

G = 1.4
RUSANOV, HLLC, EXACT, PHYS = 0, 1, 2, 3


def cons(r, u, v, p):
    return np.array([r, r * u, r * v, p / (G - 1.0) + 0.5 * r * (u * u + v * v)])


def _states(n, seed):
    rng = np.random.default_rng(seed)
    for _ in range(n):
        a = rng.uniform(0, 2 * np.pi)
        L = cons(rng.uniform(0.2, 2), rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(0.2, 2))
        R = cons(rng.uniform(0.2, 2), rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(0.2, 2))
        yield L, R, np.cos(a), np.sin(a)


def _rotate(U, t):
    c, s = np.cos(t), np.sin(t)
    return np.array([U[0], c * U[1] - s * U[2], s * U[1] + c * U[2], U[3]])


@pytest.mark.parametrize("kind", [RUSANOV, HLLC, EXACT])
def test_consistency(kind):
    for L, _, nx, ny in _states(300, 1):
        F = port.flux(kind, L, L, nx, ny, G, 1e-12, 50)
        P = port.flux(PHYS, L, L, nx, ny, G)
        assert np.allclose(F, P, rtol=1e-12, atol=1e-13 * np.abs(P).max())


@pytest.mark.parametrize("kind", [RUSANOV, HLLC, EXACT])
def test_conservation_from_both_sides(kind):
    for L, R, nx, ny in _states(300, 2):
        a = port.flux(kind, L, R, nx, ny, G, 1e-12, 50)
        b = port.flux(kind, R, L, -nx, -ny, G, 1e-12, 50)
        assert np.allclose(a, -b, rtol=1e-11, atol=1e-12 * np.abs(a).max())


@pytest.mark.parametrize("kind", [RUSANOV, HLLC, EXACT])
def test_rotational_invariance(kind):
    for i, (L, R, nx, ny) in enumerate(_states(300, 3)):
        t = 0.37 + 0.1 * i
        F = port.flux(kind, L, R, nx, ny, G, 1e-12, 50)
        n2 = _rotate(np.array([0.0, nx, ny, 0.0]), t)
        F2 = port.flux(kind, _rotate(L, t), _rotate(R, t), n2[1], n2[2], G, 1e-12, 50)
        assert np.allclose(F2, _rotate(F, t), rtol=1e-11, atol=1e-12 * np.abs(F).max())


def test_sod_interface_flux():
    L, R = cons(1.0, 0.0, 0.0, 1.0), cons(0.125, 0.0, 0.0, 0.1)
    rs, us, ps = 0.42632, 0.92745, 0.30313
    star = port.flux(PHYS, cons(rs, us, 0.0, ps), cons(rs, us, 0.0, ps), 1.0, 0.0, G)
    F = port.flux(EXACT, L, R, 1.0, 0.0, G, 1e-12, 50)
    np.testing.assert_allclose(F, star, rtol=2e-4)
    assert abs(F[2]) < 1e-15  # no tangential momentum flux
    H = port.flux(HLLC, L, R, 1.0, 0.0, G)
    assert abs(H[0] - F[0]) < 0.1 * F[0]
