"""Host-side agglomeration of the multigrid's coarse levels (CPU).

fv_mesh_agglomerate exposes the first coarse level that fv_solver_multigrid
builds (csrc/mesh_host.cpp:agglomerate).  Its checks need no GPU:

- the agglomerates partition the fine cells, each is connected through
  interior fine faces, and they hold 1-6 cells (about 4 on average);
- a coarse cell's volume and centroid are the sum and the volume-weighted
  mean of its fine cells;
- each coarse face joins two adjacent agglomerates (or one and a patch)
  and carries the summed n A of the fine faces it merges, so every coarse
  cell is closed (its outward n A sum to zero) and each patch's boundary
  n A matches the fine mesh's;
- agglomerates of a batched mesh never cross instances;
- the result is deterministic.
"""
import ctypes as C

import numpy as np
import pytest

from finitevolume_gb300 import capi, meshgen, solvers as S

MESHES = {
    "ogrid": lambda: meshgen.naca_ogrid(64, 32),
    "mixed": lambda: meshgen.naca_mixed(64, 32, seed=0),
    "triangles": lambda: meshgen.sod_strip(40, 10),
    "wavy": lambda: meshgen.wavy_quads(12, 0.03),
}


def _fine(mesh):
    ex = mesh.export()
    fi, fd, cd = ex["faces_i32"], ex["faces_f64"], ex["cells_f64"]
    return fi[:, 2], fi[:, 3], fi[:, 4], fd[:, 0] * fd[:, 2], fd[:, 1] * fd[:, 2], cd


def _components(n, edges):
    parent = np.arange(n)

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    for a, b in edges:
        ra, rb = find(a), find(b)
        if ra != rb:
            parent[ra] = rb
    return np.array([find(x) for x in range(n)])


@pytest.fixture(scope="module", params=sorted(MESHES))
def case(request):
    mesh = S.Mesh(MESHES[request.param]())
    return mesh, mesh.agglomerate()


def test_agglomerates_partition_connected(case):
    mesh, co = case
    agg = co["agg"]
    nc = co["cells_f64"].shape[0]
    assert agg.min() == 0 and agg.max() == nc - 1
    size = np.bincount(agg, minlength=nc)
    assert size.min() >= 1 and size.max() <= 6
    assert mesh.n_cells / nc >= 3.0
    L, R, _, _, _, _ = _fine(mesh)
    inside = (R >= 0) & (agg[L] == agg[np.maximum(R, 0)])
    comp = _components(mesh.n_cells, zip(L[inside], R[inside]))
    # every agglomerate is one connected component of its own cells
    for a in range(nc):
        assert np.unique(comp[agg == a]).size == 1


def test_coarse_volumes_and_centroids(case):
    mesh, co = case
    agg, cc = co["agg"], co["cells_f64"]
    _, _, _, _, _, cd = _fine(mesh)
    vol = np.bincount(agg, weights=cd[:, 0])
    np.testing.assert_allclose(cc[:, 0], vol, rtol=1e-13)
    np.testing.assert_allclose(cc[:, 1], np.bincount(agg, weights=cd[:, 0] * cd[:, 1]) / vol, rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(cc[:, 2], np.bincount(agg, weights=cd[:, 0] * cd[:, 2]) / vol, rtol=1e-12, atol=1e-13)


def test_coarse_faces_close_every_cell_and_keep_boundary(case):
    mesh, co = case
    agg, fi, fd = co["agg"], co["faces_i32"], co["faces_f64"]
    nc = co["cells_f64"].shape[0]
    cl, cr, cp = fi[:, 0], fi[:, 1], fi[:, 2]
    assert ((cr < 0) == (cp >= 0)).all()
    assert (cl[cr >= 0] < cr[cr >= 0]).all()
    nAx, nAy = fd[:, 0] * fd[:, 2], fd[:, 1] * fd[:, 2]
    # closure: outward n A of each coarse cell sums to zero
    sx = np.bincount(cl, weights=nAx, minlength=nc) - np.bincount(cr[cr >= 0], weights=nAx[cr >= 0], minlength=nc)
    sy = np.bincount(cl, weights=nAy, minlength=nc) - np.bincount(cr[cr >= 0], weights=nAy[cr >= 0], minlength=nc)
    perim = np.bincount(cl, weights=fd[:, 2], minlength=nc) + np.bincount(cr[cr >= 0], weights=fd[cr >= 0, 2],
                                                                         minlength=nc)
    assert (np.hypot(sx, sy) <= 1e-12 * perim).all()
    # each interior coarse face joins agglomerates that share a fine face
    L, R, P, fx, fy, _ = _fine(mesh)
    pairs = {(min(a, b), max(a, b)) for a, b in zip(agg[L[R >= 0]], agg[R[R >= 0]]) if a != b}
    assert pairs == {(int(a), int(b)) for a, b in zip(cl[cr >= 0], cr[cr >= 0])}
    # boundary n A per patch is the fine mesh's
    for p in np.unique(P[R < 0]):
        fine = np.array([fx[(R < 0) & (P == p)].sum(), fy[(R < 0) & (P == p)].sum()])
        coarse = np.array([nAx[cp == p].sum(), nAy[cp == p].sum()])
        np.testing.assert_allclose(coarse, fine, rtol=1e-12, atol=1e-12 * fd[cp == p, 2].sum())


def test_agglomeration_is_deterministic(case):
    mesh, co = case
    again = mesh.agglomerate()
    for k in co:
        assert np.array_equal(co[k], again[k])


def test_batched_agglomerates_stay_within_instances():
    meshes = [S.Mesh(meshgen.naca_ogrid(ni, nj)) for ni, nj in ((32, 16), (48, 24), (24, 12))]
    bm = S._BatchMesh(meshes)
    n = np.zeros(2, np.int32)
    agg = np.zeros(bm.n_cells, np.int32)
    capi.check(capi.lib().fv_mesh_agglomerate(bm.handle, capi.i32ptr(n), capi.i32ptr(agg), C.POINTER(C.c_double)(),
                                              C.POINTER(C.c_int32)(), C.POINTER(C.c_double)()))
    owner = np.repeat(np.arange(len(meshes)), np.diff(bm.offsets))
    for a in np.unique(agg):
        assert np.unique(owner[agg == a]).size == 1
    # contiguous agglomerate ranges per instance
    first = [agg[bm.offsets[i]:bm.offsets[i + 1]].min() for i in range(len(meshes))]
    last = [agg[bm.offsets[i]:bm.offsets[i + 1]].max() for i in range(len(meshes))]
    assert all(last[i] < first[i + 1] for i in range(len(meshes) - 1))


def test_agglomerate_rejects_null_counts():
    mesh = S.Mesh(meshgen.wavy_quads(4))
    st = capi.lib().fv_mesh_agglomerate(mesh.handle, C.POINTER(C.c_int32)(), C.POINTER(C.c_int32)(),
                                        C.POINTER(C.c_double)(), C.POINTER(C.c_int32)(), C.POINTER(C.c_double)())
    assert st == capi.FV_ERR_BAD_ARG
