"""Mesh generators: valid CCW cells, expected counts, FVMESH round trip."""
import os

import numpy as np

from finitevolume_gb300 import fvmesh, meshgen, solvers


def test_naca_ogrid_counts_and_validity():
    m = meshgen.naca_ogrid(256, 128)
    m.validate_ccw()
    assert m.n_cells == 32768
    mesh = solvers.Mesh(m)
    assert mesh.n_faces == 65792 and mesh.n_bfaces == 512


def test_mixed_mesh_small_is_valid_polygonal():
    m = meshgen.naca_mixed(128, 64, r_core=2.0, lloyd_iters=2, seed=3)
    m.validate_ccw()
    sizes = m.cell_sizes()
    assert sizes.min() >= 3 and (sizes >= 6).sum() > 0.2 * m.n_cells
    mesh = solvers.Mesh(m)  # the library's validation (incl. self-intersection) passes
    assert mesh.n_cells == m.n_cells


def test_sod_strip_counts():
    m = meshgen.sod_strip(50, 4)
    m.validate_ccw()
    assert m.n_cells == 400


def test_fvmesh_round_trip(tmp_path):
    m = meshgen.sod_strip(20, 3, seed=5)
    p = os.path.join(tmp_path, "s.fvmesh")
    fvmesh.write_fvmesh(m, p)
    r = fvmesh.read_fvmesh(p)
    assert np.array_equal(r.nodes, m.nodes)
    assert np.array_equal(r.cell_nodes, m.cell_nodes)
    assert r.patch_names == m.patch_names
