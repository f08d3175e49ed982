"""Launch-shape autotuner (fv_solver_autotune / fv_solver_set_launch).

The launch shape only changes how cells and faces are grouped into
blocks, never a cell's or a face's own arithmetic: after the tuner has
timed its trial steps and restored the state, a tuned solver must produce
exactly the fields of an untuned one.
"""
import numpy as np
import pytest

from finitevolume_gb300 import capi, meshgen, solvers as S
from helpers import GAMMA

pytestmark = pytest.mark.gpu


def _solver(mesh, fp32=False):
    fs = (1.0, 0.7 * np.cos(0.03), 0.7 * np.sin(0.03), 1.0 / GAMMA)
    bcs = [S.EulerBoundaryCondition(S.EulerBoundaryType.Wall),
           S.EulerBoundaryCondition(S.EulerBoundaryType.CharacteristicFarfield, S.from_primitive(*fs, GAMMA))]
    ic = S.EulerInitialCondition(S.EulerICMode.Freestream, rho=fs[0], u=fs[1], v=fs[2], p=fs[3])
    return S.EulerFVMSolver(mesh, bcs, GAMMA, 1.2, ic, S.NumericalFluxScheme.HLLC, order=2, rk_stages=3,
                            local_dt=True, fp32_flux=fp32)


@pytest.mark.parametrize("fp32", [False, True])
def test_autotune_keeps_the_state_and_the_results(gpu, fp32):
    mesh = S.Mesh(meshgen.naca_ogrid(96, 48))
    a, b = _solver(mesh, fp32), _solver(mesh, fp32)
    a.run(50)
    b.run(50)
    before = b.field().copy()
    shapes = b.autotune(steps=3, cache=False)
    assert {shapes["gradients"], shapes["faces"], shapes["cells"]} <= {128, 256, 512}
    assert np.array_equal(b.field(), before)
    a.run(40)
    b.run(40)
    assert np.array_equal(a.field(), b.field())
    np.testing.assert_allclose(a.residual().as_array(), b.residual().as_array(), rtol=1e-13)


def test_every_launch_shape_gives_the_same_fields(gpu):
    mesh = S.Mesh(meshgen.naca_ogrid(64, 32))
    ref = _solver(mesh)
    ref.run(30)
    for shape in [(128, 512, 256), (512, 128, 128), (256, 256, 512)]:
        s = _solver(mesh)
        s.set_launch(*shape)
        s.run(30)
        assert np.array_equal(s.field(), ref.field())


def test_bad_launch_shapes_are_rejected(gpu):
    s = _solver(S.Mesh(meshgen.naca_ogrid(32, 16)))
    for bad in [(64, 256, 256), (256, 1024, 256), (256, 256, 200)]:
        with pytest.raises(capi.FVError):
            s.set_launch(*bad)


def test_batch_autotune_keeps_instances(gpu):
    meshes = [S.Mesh(meshgen.naca_ogrid(32 + 8 * i, 16 + 4 * i)) for i in range(3)]
    fss = [(1.0, 0.5, 0.02, 1.0 / GAMMA)] * 3
    kinds = [S.EulerBoundaryType.Wall, S.EulerBoundaryType.CharacteristicFarfield]
    a, b = S.BatchSolver(meshes, kinds, fss), S.BatchSolver(meshes, kinds, fss)
    a.run(20)
    b.run(20)
    b.autotune(steps=2, cache=False)
    act, it, _ = b.status()
    assert (it == 20).all()
    a.run(10)
    b.run(10)
    for i in range(3):
        assert np.array_equal(a.field(i), b.field(i))
