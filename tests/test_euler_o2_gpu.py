"""GPU parity of the second-order / multi-stage path against the oracle.

The oracle (oracle/fv_oracle.cpp) is the CPU FP64 definition of the new
functionality: MUSCL reconstruction of primitive variables with LSQ or
Green-Gauss gradients and Barth-Jespersen / Venkatakrishnan limiting,
SSP-RK3, local time stepping dt_i = CFL V_i / sum_f lambda_f A_f, and the
characteristic farfield.  FP64 kernels must match it within 1e-10 relative
(fields) after hundreds of iterations; the FP32-flux mode is compared with
the FP64 GPU solve (tolerances stated per test).
"""
import numpy as np
import pytest

from finitevolume_gb300 import meshgen
from helpers import GAMMA, cons, gpu_solver, rel_err
from oracle import port

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _airfoil(M, aoa_deg, mesh):
    a = np.radians(aoa_deg)
    fs = (1.0, M * np.cos(a), M * np.sin(a), 1.0 / GAMMA)
    bcs = [(0, [0.0] * 4), (3, cons(*fs))]
    ic = {"mode": "free", "rho": fs[0], "u": fs[1], "v": fs[2], "p": fs[3]}
    return bcs, ic, fs


def _pair(mesh, bcs, ic, flux, steps, cfl, order=2, rk=3, local=True, grad=0, lim=2, k=5.0, reorder="morton"):
    fid = {"rusanov": 0, "hllc": 1, "exact": 2}[flux]
    s = gpu_solver(mesh, bcs, ic, flux, cfl=cfl, reorder=reorder, order=order, rk_stages=rk, local_dt=local,
                   gradient=grad, limiter=lim, venkat_k=k)
    o = port.OracleEuler(port.OracleMesh(mesh), bcs, gamma=GAMMA, cfl=cfl, ic=ic, flux=fid, order=order, rk=rk,
                         local_dt=local, gradient=grad, limiter=lim, venkat_k=k)
    hs = s.run(steps, history=True)
    ho = o.run(steps)
    return s, o, hs, ho


@pytest.mark.parametrize("grad,lim", [(0, 2), (0, 1), (1, 2), (0, 0)])
def test_o2_rk3_transonic_vs_oracle(gpu, grad, lim):
    mesh = meshgen.naca_ogrid(64, 32)
    bcs, ic, _ = _airfoil(0.8, 1.25, mesh)
    s, o, hs, ho = _pair(mesh, bcs, ic, "hllc", 300, 1.2, grad=grad, lim=lim)
    assert rel_err(s.field(), o.field()) < TOL
    np.testing.assert_allclose(hs, ho, rtol=1e-9)


@pytest.mark.parametrize("flux", ["rusanov", "exact"])
def test_o2_other_fluxes_vs_oracle(gpu, flux):
    mesh = meshgen.naca_ogrid(64, 32)
    bcs, ic, _ = _airfoil(0.5, 2.0, mesh)
    s, o, hs, ho = _pair(mesh, bcs, ic, flux, 150, 1.2)
    assert rel_err(s.field(), o.field()) < TOL
    np.testing.assert_allclose(hs, ho, rtol=1e-9)


def test_o2_global_dt_forward_euler_vs_oracle(gpu):
    mesh = meshgen.naca_ogrid(64, 32)
    bcs, ic, _ = _airfoil(0.5, 2.0, mesh)
    s, o, hs, ho = _pair(mesh, bcs, ic, "hllc", 100, 0.3, rk=1, local=False)
    assert rel_err(s.field(), o.field()) < TOL
    np.testing.assert_allclose(hs, ho, rtol=1e-9)


def test_o1_rk3_vs_oracle(gpu):
    mesh = meshgen.naca_ogrid(64, 32)
    bcs, ic, _ = _airfoil(0.5, 2.0, mesh)
    s, o, hs, ho = _pair(mesh, bcs, ic, "rusanov", 200, 1.5, order=1)
    assert rel_err(s.field(), o.field()) < TOL
    np.testing.assert_allclose(hs, ho, rtol=1e-9)


def test_o2_mixed_polygon_mesh_vs_oracle(gpu):
    mesh = meshgen.naca_mixed(128, 64, r_core=2.0, lloyd_iters=2, seed=0)
    bcs, ic, _ = _airfoil(0.8, 1.25, mesh)
    s, o, hs, ho = _pair(mesh, bcs, ic, "hllc", 200, 1.2, reorder="rcm")
    assert rel_err(s.field(), o.field()) < TOL
    np.testing.assert_allclose(hs, ho, rtol=1e-9)


def test_o2_sod_triangles_vs_oracle(gpu):
    mesh = meshgen.sod_strip(200, 6, seed=2)
    bcs = [(0, [0.0] * 4), (2, [0.0] * 4), (0, [0.0] * 4), (2, [0.0] * 4)]
    ic = {"mode": "two", "rho_l": 1.0, "u_l": 0.0, "v_l": 0.0, "p_l": 1.0, "rho_r": 0.125, "u_r": 0.0, "v_r": 0.0,
          "p_r": 0.1, "x0": 0.5}
    s, o, hs, ho = _pair(mesh, bcs, ic, "hllc", 150, 0.4, local=False)
    assert rel_err(s.field(), o.field()) < TOL
    np.testing.assert_allclose(hs, ho, rtol=1e-9)


def test_fp32_flux_close_to_fp64(gpu):
    """FP32 flux/gradient arithmetic, FP64 accumulation and update: the
    state stays within 1e-4 relative of the FP64 GPU solve and CL/CD within
    1e-4 absolute after 500 iterations of a transonic case."""
    mesh = meshgen.naca_ogrid(64, 32)
    bcs, ic, fs = _airfoil(0.8, 1.25, mesh)
    kw = dict(cfl=1.2, order=2, rk_stages=3, local_dt=True)
    a = gpu_solver(mesh, bcs, ic, "hllc", **kw)
    b = gpu_solver(mesh, bcs, ic, "hllc", fp32_flux=True, **kw)
    a.run(500)
    b.run(500)
    assert rel_err(b.field(), a.field()) < 1e-4
    ref = (1.0, fs[1], fs[2], fs[3], 1.0, 0.25, 0.0)
    fa, fb = a.wall_forces(*ref), b.wall_forces(*ref)
    assert abs(fa["cl"] - fb["cl"]) < 1e-4 and abs(fa["cd_total"] - fb["cd_total"]) < 1e-4
