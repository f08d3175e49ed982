"""Corrupted meshes are rejected on the host before anything reaches a GPU
(CPU).  The reference rejects them at load (src/MeshReader.cpp:125-288,
:407-443); here each corruption is planted in an otherwise valid mesh and
the library must answer with a status and a message, never a crash:
non-finite node, out-of-range node index, a cell with fewer than three
vertices, an edge shared by three cells, zero area, self-intersection, an
out-of-range patch index, and, through the face-based constructor, a face
with an out-of-range cell, a cell that lists a face it does not bound, and
a zero-volume cell.
"""
import ctypes as C

import numpy as np
import pytest

from finitevolume_gb300 import capi, meshgen, solvers
from finitevolume_gb300.fvmesh import PolyMesh


def _poly(n=3):
    return meshgen.cartesian(n, n)


def _expect_bad(poly, status=capi.FV_ERR_BAD_MESH, words=()):
    with pytest.raises(capi.FVError) as e:
        solvers.Mesh(poly)
    assert e.value.status == status
    msg = str(e.value)
    for w in words:
        assert w in msg, msg


def _copy(p):
    return PolyMesh(p.nodes.copy(), p.cell_off.copy(), p.cell_nodes.copy(), p.bedges.copy(), p.bpatch.copy(),
                    list(p.patch_names))


def test_non_finite_node():
    p = _copy(_poly())
    p.nodes[5, 1] = np.nan
    _expect_bad(p, words=("non-finite",))


def test_node_index_out_of_range():
    p = _copy(_poly())
    p.cell_nodes[2] = p.nodes.shape[0] + 7
    _expect_bad(p, words=("out-of-range node",))


def test_cell_with_two_vertices():
    p = _poly(2)
    # cell 0 keeps two of its four vertices
    off = p.cell_off.copy()
    cn = np.concatenate([p.cell_nodes[:2], p.cell_nodes[4:]])
    off = np.concatenate([[0], off[1:] - 2])
    _expect_bad(PolyMesh(p.nodes.copy(), off, cn, p.bedges.copy(), p.bpatch.copy(), list(p.patch_names)),
                words=("fewer than 3",))


def test_edge_shared_by_three_cells():
    p = _poly(2)
    # a third cell on top of cell 0
    extra = p.cell_nodes[0:4]
    off = np.concatenate([p.cell_off, [p.cell_off[-1] + 4]])
    cn = np.concatenate([p.cell_nodes, extra])
    _expect_bad(PolyMesh(p.nodes.copy(), off, cn, p.bedges.copy(), p.bpatch.copy(), list(p.patch_names)),
                words=("more than two cells",))


def test_zero_area_cell():
    p = _copy(_poly(2))
    a, b, c, d = p.cell_nodes[0:4]
    p.nodes[c] = p.nodes[b]  # collapse one edge ...
    p.nodes[d] = p.nodes[a]  # ... and the opposite one: zero area
    with pytest.raises(capi.FVError) as e:
        solvers.Mesh(p)
    assert e.value.status in (capi.FV_ERR_BAD_MESH, capi.FV_ERR_BAD_ARG)


def test_self_intersecting_cell():
    # a bow-tie quad with positive net area is still rejected
    nodes = np.array([[0.0, 0.0], [2.0, 0.0], [0.0, 1.0], [2.0, 1.5], [1.0, 3.0]])
    off = np.array([0, 4])
    cn = np.array([0, 1, 2, 3])
    be = np.array([[0, 1], [1, 2], [2, 3], [3, 0]])
    with pytest.raises(capi.FVError) as e:
        solvers.Mesh(PolyMesh(nodes, off, cn, be, np.zeros(4, np.int32), ["wall"]))
    assert e.value.status == capi.FV_ERR_BAD_MESH


def test_patch_index_out_of_range():
    p = _copy(_poly())
    p.bpatch[0] = 9
    _expect_bad(p, status=capi.FV_ERR_BAD_ARG, words=("patch index",))


def _faces_of(poly):
    ex = solvers.Mesh(poly).export()
    return ex, poly


def _create_faces(poly, fi, cf_off, cf, cd):
    h = C.c_void_p()
    nodes = np.ascontiguousarray(poly.nodes, np.float64)
    fn = np.ascontiguousarray(fi[:, 0:2], np.int32)
    fc = np.ascontiguousarray(fi[:, 2:4], np.int32)
    fp = np.ascontiguousarray(fi[:, 4], np.int32)
    st = capi.lib().fv_mesh_create_faces(nodes.shape[0], capi.dptr(nodes), fi.shape[0], capi.i32ptr(fn),
                                         capi.i32ptr(fc), capi.i32ptr(fp), cd.shape[0], capi.i32ptr(cf_off),
                                         capi.i32ptr(cf), capi.dptr(np.ascontiguousarray(cd)),
                                         len(poly.patch_names), 0, C.byref(h))
    if st == capi.FV_OK:
        capi.lib().fv_mesh_destroy(h)
    return st


def test_face_constructor_accepts_the_exported_mesh():
    ex, poly = _faces_of(_poly())
    assert _create_faces(poly, ex["faces_i32"], ex["cell_face_off"], ex["cell_faces"], ex["cells_f64"]) == capi.FV_OK


@pytest.mark.parametrize("how", ["cell_index", "foreign_face", "zero_volume"])
def test_face_constructor_rejects_corruption(how):
    ex, poly = _faces_of(_poly())
    fi, off, cf, cd = ex["faces_i32"].copy(), ex["cell_face_off"].copy(), ex["cell_faces"].copy(), ex["cells_f64"].copy()
    if how == "cell_index":
        fi[0, 2] = cd.shape[0] + 3
    elif how == "foreign_face":
        # cell 0 lists a face of the last cell instead of its own
        last = cf[off[-2]:off[-1]]
        own = set(cf[off[0]:off[1]].tolist())
        cf[off[0]] = next(int(f) for f in last if int(f) not in own)
    else:
        cd[4, 0] = 0.0
    assert _create_faces(poly, fi, off, cf, cd) in (capi.FV_ERR_BAD_MESH, capi.FV_ERR_BAD_ARG)
    assert capi.lib().fv_last_error()
