"""The dataflow form's partition (host side, no GPU): the plan that the
persistent first-order kernel's local-dt form runs on
(Solver::build_dataflow, exposed as fv_mesh_dataflow_plan).

Its correctness rests on the dependency lists: a block's face phase of
step s reads the step-s states of its faces' right cells, so it must wait
for the cell phase of step s-1 of their owners; a block's cell phase reads
the fluxes of every face of its cells and overwrites the states that those
faces' owners read, so it must wait for their face phase of step s.  The
tests check, on O-grids in three cell orders and on a mixed mesh, that:

- the cell ranges cover the mesh in whole 32-cell warps (the norm partials
  are formed per warp and folded in the tiles of the two-kernel path);
- every face belongs to the block owning its left cell, boundary faces
  first in each block's range;
- every face between two blocks puts the right cell's owner in the left
  owner's face-phase list and the left owner in the right owner's
  cell-phase list, and no list holds anything else (sorted, unique, no
  self-dependency);
- the plan is used (no list longer than 32 blocks) on the Morton-ordered
  meshes, and the blocks holding characteristic-farfield faces get no more
  cells than the others.

No reference counterpart (the reference's loops are OpenMP).
"""
import numpy as np
import pytest

from finitevolume_gb300 import capi, meshgen, solvers as S

WALL, CHAR = 0, 3


def _check(plan, n_cells):
    nb = plan["nb"]
    co, fo, faces, fc = plan["cell_off"], plan["face_off"], plan["faces"], plan["face_cells"]
    F = fc.shape[0]
    assert co[0] == 0 and co[nb] == n_cells and np.all(np.diff(co) >= 0)
    assert np.all(co[:nb] % 32 == 0)
    owner = np.searchsorted(co, np.arange(n_cells), side="right") - 1
    assert fo[0] == 0 and fo[nb] == F and np.array_equal(np.sort(faces), np.arange(F))
    for b in range(nb):
        fb = faces[fo[b]:fo[b + 1]]
        assert np.all(owner[fc[fb, 0]] == b)
        bnd = fc[fb, 1] < 0
        # boundary faces first
        assert not np.any(bnd[1:] & ~bnd[:-1])
    # dependencies: exactly the block pairs that share a face
    want_f = [set() for _ in range(nb)]
    want_c = [set() for _ in range(nb)]
    inner = fc[:, 1] >= 0
    a = owner[fc[inner, 0]]
    r = owner[fc[inner, 1]]
    for x, y in zip(a[a != r], r[a != r]):
        want_f[x].add(int(y))
        want_c[y].add(int(x))
    for b in range(nb):
        df = plan["dep_face"][plan["dep_face_off"][b]:plan["dep_face_off"][b + 1]]
        dc = plan["dep_cell"][plan["dep_cell_off"][b]:plan["dep_cell_off"][b + 1]]
        assert list(df) == sorted(want_f[b]) and list(dc) == sorted(want_c[b])
        assert b not in want_f[b] and b not in want_c[b]
    return owner


@pytest.mark.parametrize("reorder", ["morton", "rcm", "none"])
@pytest.mark.parametrize("size", [(64, 32), (256, 128), (512, 256)])
def test_plan_covers_every_dependency(reorder, size):
    m = S.Mesh(meshgen.naca_ogrid(*size), reorder=reorder)
    plan = m.dataflow_plan([WALL, CHAR], blocks=152)
    assert plan["nb"] == min(152, (m.n_cells + 31) // 32)
    _check(plan, m.n_cells)
    if reorder == "morton":
        assert plan["used"]


def test_plan_on_a_mixed_mesh():
    m = S.Mesh(meshgen.naca_mixed(128, 64), reorder="morton")
    plan = m.dataflow_plan([WALL, CHAR], blocks=152)
    _check(plan, m.n_cells)
    assert plan["used"]


def test_farfield_blocks_get_fewer_cells():
    # config 1's mesh: the farfield ghost state is the longest chain of the
    # face phase, so the blocks holding those faces are given fewer cells
    m = S.Mesh(meshgen.naca_ogrid(256, 128), reorder="morton")
    plan = m.dataflow_plan([WALL, CHAR], blocks=152)
    owner = _check(plan, m.n_cells)
    fc = plan["face_cells"]
    e = m.export()
    far = np.zeros(plan["nb"], bool)
    # patch of each device face: the face ids of the plan are device ids;
    # boundary faces on patch 1 are the farfield (the O-grid's outer ring)
    bnd = fc[:, 1] < 0
    cells = np.diff(plan["cell_off"])
    radius = np.hypot(*(e["cells_f64"][m.permutation()][:, 1:3].T))
    outer = bnd & (radius[fc[:, 0]] > 5.0)
    far[np.unique(owner[fc[outer, 0]])] = True
    assert far.any() and (~far).any()
    assert cells[far].max() <= cells[~far].max()
    assert cells[far].mean() < cells[~far].mean()
    # the same mesh with a slip wall all round is split evenly
    even = m.dataflow_plan([WALL, WALL], blocks=152)
    assert np.diff(even["cell_off"]).min() >= 192


def test_plan_rejects_bad_arguments():
    m = S.Mesh(meshgen.naca_ogrid(64, 32))
    with pytest.raises(capi.FVError):
        m.dataflow_plan([WALL, CHAR], blocks=0)
    with pytest.raises(capi.FVError):
        m.dataflow_plan([WALL, 9], blocks=152)
