"""GPU parity of the first-order Euler path against the reference's outputs.

Strict kernels (no FMA contraction) must reproduce the reference's fields
bit for bit for the Rusanov and HLLC fluxes (the exact Riemann solver calls
pow(), whose last bit differs between CUDA and glibc); the default kernels
must agree within 1e-10 relative.  Residual histories: 1e-10 relative (the
sums are reductions in a different order).
"""
import numpy as np
import pytest

from finitevolume_gb300 import capi, meshgen
from helpers import (GAMMA, case_of, cons, gpu_solver, load_golden, parse_bcs, parse_ic, poly_of, rel_err)
from oracle import port

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _run_golden(name, flux, strict, reorder="morton"):
    g = load_golden(name)
    case = case_of(g)
    poly = poly_of(g)
    s = gpu_solver(poly, parse_bcs(case["bc"], poly.patch_names), parse_ic(case["ic"]), flux, cfl=case["cfl"],
                   reorder=reorder, strict=strict)
    hist = s.run(case["steps"], history=True)
    return s, hist, g[f"field_{flux}"], g[f"hist_{flux}"]


@pytest.mark.parametrize("name", ["naca_og64", "sod_tri"])
@pytest.mark.parametrize("flux", ["rusanov", "hllc"])
def test_strict_bitwise_vs_reference(gpu, name, flux):
    s, hist, ref_field, ref_hist = _run_golden(name, flux, strict=True)
    assert np.array_equal(s.field(), ref_field)
    np.testing.assert_allclose(hist, ref_hist, rtol=TOL)


@pytest.mark.parametrize("name", ["naca_og64", "sod_tri"])
@pytest.mark.parametrize("flux", ["rusanov", "hllc", "exact"])
def test_fast_within_tolerance_vs_reference(gpu, name, flux):
    s, hist, ref_field, ref_hist = _run_golden(name, flux, strict=False)
    assert rel_err(s.field(), ref_field) < TOL
    np.testing.assert_allclose(hist, ref_hist, rtol=TOL)


def test_exact_strict_within_tolerance(gpu):
    s, hist, ref_field, ref_hist = _run_golden("naca_og64", "exact", strict=True)
    assert rel_err(s.field(), ref_field) < TOL


@pytest.mark.parametrize("reorder", ["none", "rcm"])
def test_layout_does_not_change_bits(gpu, reorder):
    s, _, ref_field, _ = _run_golden("sod_tri", "hllc", strict=True, reorder=reorder)
    assert np.array_equal(s.field(), ref_field)


def test_step_and_run_agree_and_residual(gpu):
    g = load_golden("naca_og64")
    case = case_of(g)
    poly = poly_of(g)
    bcs, ic = parse_bcs(case["bc"], poly.patch_names), parse_ic(case["ic"])
    a = gpu_solver(poly, bcs, ic, "hllc", strict=True)
    b = gpu_solver(poly, bcs, ic, "hllc", strict=True)
    for _ in range(7):
        a.step()
    b.run(7)
    assert np.array_equal(a.field(), b.field())
    r = a.residual().as_array()
    np.testing.assert_allclose(r, g["hist_hllc"][6], rtol=TOL)
    assert a.gas_gamma() == GAMMA


def test_set_field_and_set_cfl_follow_oracle(gpu):
    g = load_golden("naca_og64")
    case = case_of(g)
    poly = poly_of(g)
    bcs, ic = parse_bcs(case["bc"], poly.patch_names), parse_ic(case["ic"])
    s = gpu_solver(poly, bcs, ic, "rusanov", strict=True)
    o = port.OracleEuler(port.OracleMesh(poly), bcs, gamma=GAMMA, cfl=0.5, ic=ic, flux=0)
    s.run(10)
    o.run(10)
    U = s.field()
    U[:, 0] *= 1.0 + 1e-3 * np.sin(np.arange(U.shape[0]))
    s.set_field(U)
    o.set_field(U)
    assert np.all(s.residual().as_array() == 0.0)
    s.set_cfl(0.3)
    o.set_cfl(0.3)
    hs = s.run(15, history=True)
    ho = o.run(15)
    assert np.array_equal(s.field(), o.field())
    np.testing.assert_allclose(hs, ho, rtol=TOL)


@pytest.mark.parametrize("flux", ["rusanov", "hllc"])
def test_local_dt_and_characteristic_farfield_vs_oracle(gpu, flux):
    poly = meshgen.naca_ogrid(64, 32)
    M, aoa = 0.5, np.radians(2.0)
    fs = (1.0, M * np.cos(aoa), M * np.sin(aoa), 1.0 / GAMMA)
    bcs = [(0, [0.0] * 4), (3, cons(*fs))]
    ic = {"mode": "free", "rho": fs[0], "u": fs[1], "v": fs[2], "p": fs[3]}
    s = gpu_solver(poly, bcs, ic, flux, strict=True, local_dt=True)
    o = port.OracleEuler(port.OracleMesh(poly), bcs, gamma=GAMMA, cfl=0.5, ic=ic, flux=1 if flux == "hllc" else 0,
                         local_dt=True)
    hs = s.run(150, history=True)
    ho = o.run(150)
    assert rel_err(s.field(), o.field()) < TOL
    np.testing.assert_allclose(hs, ho, rtol=1e-9)


def test_wall_forces_match_oracle(gpu):
    g = load_golden("naca_og64")
    case = case_of(g)
    poly = poly_of(g)
    bcs, ic = parse_bcs(case["bc"], poly.patch_names), parse_ic(case["ic"])
    s = gpu_solver(poly, bcs, ic, "hllc")
    s.run(200)
    o = port.OracleEuler(port.OracleMesh(poly), bcs, gamma=GAMMA, cfl=0.5, ic=ic, flux=1)
    o.run(200)
    ref = [1.0, ic["u"], ic["v"], ic["p"], 1.0, 0.25, 0.0]
    f = s.wall_forces(*ref)
    fo = o.wall_forces([1 if t == 0 else 0 for t, _ in bcs], np.array(ref))
    keys = ["friction_drag", "pressure_drag", "total_drag", "lift", "moment", "cd_friction", "cd_pressure",
            "cd_total", "cl", "cm", "n_wall_faces"]
    for i, k in enumerate(keys):
        assert abs(f[k] - fo[i]) <= 1e-10 * max(1.0, abs(fo[i])), k
    assert f["n_wall_faces"] == 64


def test_nonfinite_state_is_reported(gpu):
    poly = meshgen.cartesian(8, 8)
    bcs = [(0, [0.0] * 4)] * 4
    s = gpu_solver(poly, bcs, {"mode": "free", "rho": 1.0, "u": 0.1, "v": 0.0, "p": 1.0}, "rusanov")
    U = s.field()
    U[5, 0] = np.nan
    s.set_field(U)
    with pytest.raises(capi.FVError) as e:
        s.run(2)
    assert e.value.status == capi.FV_ERR_NONFINITE
