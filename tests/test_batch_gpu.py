"""Batched steady solves (one launch sequence for many meshes).

Each instance of a batch must evolve exactly as a standalone solve of the
same case (same kernels, same per-cell arithmetic: the fields agree to
1e-12 relative), and an instance whose density residual falls below the
tolerance must be frozen while the others continue (per-instance early exit).
"""
import numpy as np
import pytest

from finitevolume_gb300 import meshgen, solvers as S
from helpers import GAMMA, rel_err

pytestmark = pytest.mark.gpu

CASES = [("2412", 32, 16, 0.5, 2.0), ("0012", 48, 24, 0.7, -1.0), ("4415", 40, 20, 0.3, 5.0)]


def _fs(M, aoa):
    a = np.radians(aoa)
    return (1.0, M * np.cos(a), M * np.sin(a), 1.0 / GAMMA)


def _meshes():
    return [S.Mesh(meshgen.naca_ogrid(ni, nj, code=code)) for code, ni, nj, _, _ in CASES]


def _standalone(mesh, fs, fp32=False):
    bcs = [S.EulerBoundaryCondition(S.EulerBoundaryType.Wall),
           S.EulerBoundaryCondition(S.EulerBoundaryType.CharacteristicFarfield, S.from_primitive(*fs, GAMMA))]
    ic = S.EulerInitialCondition(S.EulerICMode.Freestream, rho=fs[0], u=fs[1], v=fs[2], p=fs[3])
    return S.EulerFVMSolver(mesh, bcs, GAMMA, 1.2, ic, S.NumericalFluxScheme.HLLC, order=2, rk_stages=3,
                            local_dt=True, fp32_flux=fp32)


@pytest.mark.parametrize("fp32", [False, True])
def test_batch_instances_match_standalone_solves(gpu, fp32):
    meshes = _meshes()
    fss = [_fs(M, a) for _, _, _, M, a in CASES]
    b = S.BatchSolver(meshes, [S.EulerBoundaryType.Wall, S.EulerBoundaryType.CharacteristicFarfield], fss,
                      fp32_flux=fp32)
    b.run(120)
    act, it, norms = b.status()
    assert act.all() and (it == 120).all()
    for i, (m, fs) in enumerate(zip(meshes, fss)):
        s = _standalone(m, fs, fp32)
        s.run(120)
        assert rel_err(b.field(i), s.field()) < 1e-12
        ref = (fs[0], fs[1], fs[2], fs[3], 1.0, 0.25, 0.0)
        fb, fa = b.wall_forces(i, *ref), s.wall_forces(*ref)
        assert abs(fb["cl"] - fa["cl"]) < 1e-12 and abs(fb["cd_total"] - fa["cd_total"]) < 1e-12
        # the batch's per-instance norm is the standalone solve's last norm
        np.testing.assert_allclose(norms[i], s.residual().as_array(), rtol=1e-10)


def test_batch_early_exit_freezes_converged_instances(gpu):
    meshes = _meshes()
    fss = [_fs(M, a) for _, _, _, M, a in CASES]
    b = S.BatchSolver(meshes, [S.EulerBoundaryType.Wall, S.EulerBoundaryType.CharacteristicFarfield], fss)
    b.run(200)
    _, _, norms = b.status()
    # freeze the instance with the smallest density residual at a level it
    # reaches within the next iterations, keep the others running
    k = int(np.argmin(norms[:, 0]))
    b.set_tolerance(norms[k, 0] * 0.98)
    b.run(300)
    act, it, _ = b.status()
    assert not act[k] and it[k] < 500
    frozen = b.field(k).copy()
    others = [i for i in range(len(CASES)) if act[i]]
    before = {i: b.field(i).copy() for i in others}
    b.run(20)
    assert np.array_equal(b.field(k), frozen)
    for i in others:
        assert not np.array_equal(b.field(i), before[i])


def test_batch_set_active_freezes_and_resumes_one_instance(gpu):
    meshes = _meshes()
    fss = [_fs(M, a) for _, _, _, M, a in CASES]
    b = S.BatchSolver(meshes, [S.EulerBoundaryType.Wall, S.EulerBoundaryType.CharacteristicFarfield], fss)
    b.run(10)
    b.set_active(1, False)
    frozen = b.field(1).copy()
    others = {i: b.field(i).copy() for i in (0, 2)}
    b.run(10)
    act, it, _ = b.status()
    assert not act[1] and it[1] == 10 and it[0] == 20
    assert np.array_equal(b.field(1), frozen)
    assert all(not np.array_equal(b.field(i), others[i]) for i in (0, 2))
    b.set_active(1, True)
    b.run(5)
    act, it, _ = b.status()
    assert act[1] and it[1] == 15
    with pytest.raises(Exception):
        b.set_active(7, False)

