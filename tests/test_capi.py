"""CPU checks of the C ABI: the library loads, exports every declared
symbol, builds meshes exactly like the reference reader, and fails loudly
(no CPU fallback) when no GPU is present."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from finitevolume_gb300 import capi, meshgen, solvers
from helpers import load_golden, poly_of

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(fv_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    L = capi.lib()
    names = declared_functions()
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(L, n), n
    assert set(capi.SIGNATURES) >= names


def declared_arity():
    """Parameter count of every prototype in include/fv_gb300.h."""
    txt = open(os.path.join(ROOT, "include", "fv_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    out = {}
    for name, params in re.findall(r"\b(fv_[a-z0-9_]+)\s*\(([^;{)]*)\)\s*;", txt):
        params = params.strip()
        out[name] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_bindings_match_the_declared_arity():
    """capi.py declares each entry point with as many arguments as the
    header's prototype (a drifted binding would pass garbage silently)."""
    arity = declared_arity()
    assert len(arity) >= 50
    for name, n in sorted(arity.items()):
        assert len(capi.SIGNATURES[name][1]) == n, (name, n, capi.SIGNATURES[name])


def test_abi_version_and_device_count():
    L = capi.lib()
    assert L.fv_abi_version() >= 100
    assert L.fv_device_count() >= 0


def test_mesh_topology_matches_reference_reader():
    g = load_golden("wavy_grad")
    m = solvers.Mesh(poly_of(g))
    ex = m.export()
    assert np.array_equal(ex["faces_i32"].ravel(), g["mesh_faces_i32"])
    assert np.array_equal(ex["faces_f64"].ravel(), g["mesh_faces_f64"])
    assert np.array_equal(ex["cells_f64"].ravel(), g["mesh_cells_f64"])
    assert np.array_equal(ex["cell_face_off"], g["mesh_cell_face_off"])
    assert np.array_equal(ex["cell_faces"], g["mesh_cell_faces"])


@pytest.mark.parametrize("reorder", ["none", "morton", "rcm"])
def test_reorder_is_a_permutation(reorder):
    m = solvers.Mesh(meshgen.naca_ogrid(32, 16), reorder=reorder)
    p = m.permutation()
    assert np.array_equal(np.sort(p), np.arange(m.n_cells))


def test_untagged_boundary_face_is_rejected():
    poly = meshgen.cartesian(3, 3)
    keep = poly.bpatch != 3  # drop the 'left' patch tags
    poly.bedges, poly.bpatch = poly.bedges[keep], poly.bpatch[keep]
    with pytest.raises(capi.FVError) as e:
        solvers.Mesh(poly)
    assert e.value.status == capi.FV_ERR_BAD_MESH


def test_clockwise_cell_is_rejected():
    poly = meshgen.cartesian(2, 2)
    poly.cell_nodes[0:4] = poly.cell_nodes[0:4][::-1].copy()
    with pytest.raises(capi.FVError) as e:
        solvers.Mesh(poly)
    assert e.value.status == capi.FV_ERR_BAD_MESH


def test_solver_without_gpu_fails_loudly():
    if capi.lib().fv_device_count() > 0:
        pytest.skip("a GPU is present")
    m = solvers.Mesh(meshgen.cartesian(2, 2))
    bcs = [solvers.EulerBoundaryCondition()] * 4
    with pytest.raises(capi.FVError) as e:
        solvers.EulerFVMSolver(m, bcs, 1.4, 0.5, solvers.EulerInitialCondition())
    assert e.value.status == capi.FV_ERR_CUDA
