"""GPU GradientCalculator / face_gradient against the reference's outputs.

The fixture (tests/golden/wavy_grad.npz) holds the reference's gradients of a
linear and a quadratic field on a non-affine quad mesh, for both schemes,
plus face_gradient's corrected normal derivative, the corrected gradient
vector and face_normal_distance for every face.  The device code keeps the
reference's evaluation order without FMA contraction: bit-identical.
"""
import numpy as np
import pytest

from finitevolume_gb300 import meshgen, solvers as S
from finitevolume_gb300.fvmesh import cell_centroids
from helpers import load_golden, poly_of

pytestmark = pytest.mark.gpu


def _poly(c, x, y):
    return c[0] + c[1] * x + c[2] * y + c[3] * x * x + c[4] * x * y + c[5] * y * y


@pytest.mark.parametrize("scheme", ["lsq", "gg"])
@pytest.mark.parametrize("field", ["lin", "quad"])
@pytest.mark.parametrize("reorder", ["morton", "rcm"])
def test_gradients_bitwise_vs_reference(gpu, scheme, field, reorder):
    g = load_golden("wavy_grad")
    poly = poly_of(g)
    mesh = S.Mesh(poly, reorder=reorder)
    ex = mesh.export()
    c = g[f"coef_{field}"]
    cxy = ex["cells_f64"][:, 1:3]
    phi = _poly(c, cxy[:, 0], cxy[:, 1])
    fd = ex["faces_f64"]
    bnd = ex["faces_i32"][:, 3] < 0
    bphi = np.where(bnd, _poly(c, fd[:, 3], fd[:, 4]), 0.0)
    calc = S.GradientCalculator(mesh, S.GradientScheme.LeastSquares if scheme == "lsq" else S.GradientScheme.GreenGauss)
    grad, fo = calc.compute(phi, bphi, face_gradients=True)
    want_g, want_f = g[f"grad_{scheme}_{field}"], g[f"facegrad_{scheme}_{field}"]
    if scheme == "lsq":
        # no libm call on this path: bit-identical on any host
        assert np.array_equal(grad, want_g)
    # Green-Gauss weights and the face geometry go through std::hypot, whose
    # last bit may differ between the host that made the fixture and this one.
    assert np.max(np.abs(grad - want_g)) <= 1e-13 * max(1.0, np.max(np.abs(want_g)))
    assert np.max(np.abs(fo - want_f), axis=0).max() <= 1e-12 * max(1.0, np.max(np.abs(want_f)))


def test_lsq_exact_for_linear_field_on_polygons(gpu):
    """--verify-gradient's property (src/main.cpp:1443-1527) on a polygon mesh."""
    poly = meshgen.naca_mixed(64, 32, r_core=2.0, lloyd_iters=1, seed=4)
    mesh = S.Mesh(poly)
    cxy = cell_centroids(poly)
    ex = mesh.export()
    phi = 0.3 + 1.7 * cxy[:, 0] - 0.6 * cxy[:, 1]
    bphi = 0.3 + 1.7 * ex["faces_f64"][:, 3] - 0.6 * ex["faces_f64"][:, 4]
    grad = S.GradientCalculator(mesh).compute(phi, bphi)
    assert np.max(np.abs(grad - np.array([1.7, -0.6]))) < 1e-9
