"""Bit-for-bit layout check: the cell ordering (identity, Morton, RCM) and
the tile sort by face count only renumber cells; every cell keeps the
reference's own face order and every face its orientation, so the
second-order solution is bit-identical in every layout (Sod shock tube on
a randomly perturbed triangle strip, global and local time steps)."""
import numpy as np
import pytest

from finitevolume_gb300 import meshgen, solvers as S
from helpers import GAMMA

pytestmark = pytest.mark.gpu


def sod_solver(poly, reorder, local_dt, fp32=False):
    mesh = S.Mesh(poly, reorder=reorder)
    bcs = [S.EulerBoundaryCondition(S.EulerBoundaryType.Wall), S.EulerBoundaryCondition(S.EulerBoundaryType.Outflow),
           S.EulerBoundaryCondition(S.EulerBoundaryType.Wall), S.EulerBoundaryCondition(S.EulerBoundaryType.Outflow)]
    ic = S.EulerInitialCondition(S.EulerICMode.TwoRegion, rho_l=1.0, u_l=0.0, v_l=0.0, p_l=1.0, rho_r=0.125, u_r=0.0,
                                 v_r=0.0, p_r=0.1, x0=0.5)
    return S.EulerFVMSolver(mesh, bcs, GAMMA, 0.5, ic, S.NumericalFluxScheme.HLLC, order=2, rk_stages=3,
                            local_dt=local_dt, fp32_flux=fp32)


@pytest.mark.parametrize("local_dt,fp32", [(False, False), (True, False), (False, True)])
def test_sod_strip_is_bitwise_layout_invariant(gpu, local_dt, fp32):
    poly = meshgen.sod_strip(200, 50, seed=4)
    fields = []
    for reorder in ("none", "morton", "rcm"):
        s = sod_solver(poly, reorder, local_dt, fp32)
        s.run(60)
        fields.append(s.field())
    assert np.array_equal(fields[0], fields[1]) and np.array_equal(fields[0], fields[2])
