"""The persistent first-order kernel (one cooperative launch per chunk of
steps, grid barriers between the face and cell phases, or with local dt
neighbour-progress waits: the dataflow form) against the two-kernel path,
and its bounded waits.

- Same fields and residual histories bit for bit as the two-kernel path in
  strict mode (Rusanov and HLLC, global dt with the fixed farfield, local dt
  with the characteristic farfield), and within 1e-10 in the default build
  (which forms 1/rho and the local-dt factor with fewer FP64 instructions).
- The dataflow form (the default with local dt) gives the same fields and
  histories as the grid-barrier form, bit for bit in strict mode, on meshes
  from 64 blocks of one cell warp each to blocks of several hundred cells
  and faces (the loops over a block's cells and faces).
- A barrier that waits for an arrival that never comes gives up after its
  cycle limit: fv_step returns FV_ERR_TIMEOUT, nothing hangs, the state is
  untouched (the first barrier precedes every update) and the solver steps
  normally once the limit is restored; in both forms.

Reference: src/EulerFVMSolver.cpp:58-162 (step, compute_dt).
"""
import numpy as np
import pytest

from finitevolume_gb300 import capi, meshgen, solvers as S
from helpers import gpu_solver, rel_err, GAMMA

pytestmark = pytest.mark.gpu


def _case(local):
    M, aoa = 0.5, np.radians(2.0)
    r, u, v, p = 1.0, M * np.cos(aoa), M * np.sin(aoa), 1.0 / GAMMA
    st = list(S.from_primitive(r, u, v, p, GAMMA))
    bcs = [(0, [0.0] * 4), (3 if local else 1, st)]
    return bcs, {"mode": "free", "rho": r, "u": u, "v": v, "p": p}


@pytest.mark.parametrize("flux", ["rusanov", "hllc"])
@pytest.mark.parametrize("local", [False, True])
@pytest.mark.parametrize("strict", [True, False])
def test_persistent_matches_two_kernel_path(gpu, flux, local, strict):
    poly = meshgen.naca_ogrid(128, 64)
    bcs, ic = _case(local)
    a = gpu_solver(poly, bcs, ic, flux, cfl=0.5, local_dt=local, strict=strict)
    b = gpu_solver(poly, bcs, ic, flux, cfl=0.5, local_dt=local, strict=strict)
    on, grid = a.persistent()
    assert on == (2 if local else 1) and grid > 0
    b.set_persistent(False)
    assert not b.persistent()[0]
    ha = a.run(300, history=True)
    hb = b.run(300, history=True)
    if strict:
        assert np.array_equal(a.field(), b.field())
        assert np.array_equal(ha, hb)
    else:
        assert rel_err(a.field(), b.field()) <= 1e-10
        np.testing.assert_allclose(ha, hb, rtol=1e-10, atol=0)
    # chunk boundaries (256 steps per launch) are invisible: 300 = 256 + 44
    c = gpu_solver(poly, bcs, ic, flux, cfl=0.5, local_dt=local, strict=strict)
    for _ in range(3):
        c.run(100)
    assert np.array_equal(c.field(), a.field())


@pytest.mark.parametrize("flux", ["rusanov", "hllc"])
@pytest.mark.parametrize("strict", [True, False])
@pytest.mark.parametrize("size", [(64, 32), (128, 64), (512, 256)])
def test_dataflow_form_matches_barrier_form(gpu, flux, strict, size):
    poly = meshgen.naca_ogrid(*size)
    bcs, ic = _case(True)
    a = gpu_solver(poly, bcs, ic, flux, cfl=0.5, local_dt=True, strict=strict)
    b = gpu_solver(poly, bcs, ic, flux, cfl=0.5, local_dt=True, strict=strict)
    b.set_persistent("barrier")
    assert a.persistent()[0] == 2 and b.persistent()[0] == 1
    n = 300 if size[0] < 512 else 60
    ha = a.run(n, history=True)
    hb = b.run(n, history=True)
    if strict:
        assert np.array_equal(a.field(), b.field())
        assert np.array_equal(ha, hb)
    else:
        assert rel_err(a.field(), b.field()) <= 1e-13
        np.testing.assert_allclose(ha, hb, rtol=1e-13, atol=0)


@pytest.mark.parametrize("strict", [True, False])
def test_exact_riemann_flux_in_both_forms(gpu, strict):
    # the exact Riemann flux (its Newton iteration and powers inside the
    # face phase): dataflow form, grid-barrier form and two-kernel path
    poly = meshgen.naca_ogrid(64, 32)
    bcs, ic = _case(True)
    runs = []
    for mode in (True, "barrier", False):
        s = gpu_solver(poly, bcs, ic, "exact", cfl=0.5, local_dt=True, strict=strict)
        s.set_persistent(mode)
        h = s.run(200, history=True)
        runs.append((s.field(), h))
    if strict:
        assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])
        assert np.array_equal(runs[0][0], runs[2][0]) and np.array_equal(runs[0][1], runs[2][1])
    else:
        assert rel_err(runs[0][0], runs[1][0]) <= 1e-13
        assert rel_err(runs[0][0], runs[2][0]) <= 1e-10
        np.testing.assert_allclose(runs[0][1], runs[2][1], rtol=1e-10, atol=0)


@pytest.mark.parametrize("local", [False, True])
def test_barrier_wait_runs_out_and_reports_timeout(gpu, local):
    poly = meshgen.naca_ogrid(64, 32)
    bcs, ic = _case(local)
    s = gpu_solver(poly, bcs, ic, "rusanov", cfl=0.5, local_dt=local)
    assert s.persistent()[0] == (2 if local else 1)
    s.run(5)
    before = s.field()
    # every barrier now waits for one more block than the grid has
    s.set_wait_limit(2_000_000, phantom_arrivals=1)
    with pytest.raises(capi.FVError) as ei:
        s.run(1)
    assert ei.value.status == capi.FV_ERR_TIMEOUT
    assert np.array_equal(s.field(), before)
    # restored: steps again, same as a solver that never timed out
    s.set_wait_limit(2_000_000_000, phantom_arrivals=0)
    s.run(3)
    ref = gpu_solver(poly, bcs, ic, "rusanov", cfl=0.5, local_dt=local)
    ref.run(8)
    assert np.array_equal(s.field(), ref.field())
