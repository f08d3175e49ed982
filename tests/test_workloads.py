"""The seeded synthetic workloads match the configurations they stand for
(CPU).  No external dataset exists; these generators produce the meshes and
flow cases of the benchmark and parity configurations, and the checks below
pin their stated shapes, sizes and value ranges:

- NACA0012 O-grid, 256 x 128 quads (32,768 cells), closed trailing edge,
  first wall spacing 1e-3 chord, farfield circle at 20 chords;
- the adjoint O-grid, 1024 x 488 quads (499,712 cells);
- the Sod strip, 1000 x 500 x 2 = 1,000,000 randomly perturbed triangles;
- the mixed mesh: an O-grid core of quads inside a Lloyd-relaxed polygonal
  region of 3-9-sided cells, more than 99.9 % of them 4-9-sided (checked
  at a reduced size);
- the NACA4412 hybrid mesh (no overlapping cells): wall-clustered quad layers (first spacing,
  growth 1.15) inside random triangles, farfield at 30 chords (reduced size);
- the 256-instance batch: camber 0-6 %, thickness 8-18 %, 4k-64k cells
  log-uniform, M 0.3-0.85, AoA -4..8 degrees.
"""
import numpy as np

from finitevolume_gb300 import meshgen


def _wall_and_far(poly, center=(0.5, 0.0)):
    r = np.hypot(*(poly.nodes - np.asarray(center)).T)
    names = list(poly.patch_names)
    be, bp = poly.bedges, poly.bpatch
    wall = np.unique(be[bp == names.index("airfoil")])
    far = np.unique(be[bp == names.index("farfield")])
    return r, wall, far


def _first_spacing(poly, wall):
    """Smallest distance from a wall node to a node that is not on the wall."""
    nodes = poly.nodes
    others = np.setdiff1d(np.arange(nodes.shape[0]), wall)
    # the first off-wall ring: nodes closest to the wall
    d = np.full(wall.size, np.inf)
    off = poly.cell_off
    for c in range(poly.n_cells):
        cn = poly.cell_nodes[off[c]:off[c + 1]]
        on = np.isin(cn, wall)
        if on.any() and (~on).any():
            for i in np.nonzero(on)[0]:
                w = np.searchsorted(wall, cn[i])
                for j in cn[~on]:
                    d[w] = min(d[w], np.hypot(*(nodes[cn[i]] - nodes[j])))
    del others
    return d[np.isfinite(d)]


def test_naca0012_ogrid_config():
    m = meshgen.naca_ogrid(256, 128)
    assert m.n_cells == 32768 and m.cell_sizes().min() == 4 and m.cell_sizes().max() == 4
    r, wall, far = _wall_and_far(m)
    assert wall.size == 256 and far.size == 256
    np.testing.assert_allclose(r[far], 20.0, rtol=1e-12)
    # closed trailing edge: a single wall node at x = 1, y = 0
    te = m.nodes[wall][np.argmax(m.nodes[wall][:, 0])]
    np.testing.assert_allclose(te, [1.0, 0.0], atol=1e-12)
    # maximum thickness 12 % of the chord
    xw, yw = m.nodes[wall].T
    upper = yw >= 0
    assert abs((yw[upper].max() - yw[~upper].min()) - 0.12) < 2e-3
    sp = _first_spacing(m, wall)
    assert abs(np.median(sp) - 1e-3) < 1e-4


def test_adjoint_ogrid_and_sod_strip_sizes():
    assert meshgen.naca_ogrid(1024, 488).n_cells == 499712
    s = meshgen.sod_strip(1000, 500)
    assert s.n_cells == 1_000_000 and s.cell_sizes().max() == 3


def test_mixed_mesh_structure():
    ni, nj = 256, 128
    m = meshgen.naca_mixed(ni, nj, first=1e-3, r_core=2.0, r_far=20.0, code="0012", lloyd_iters=4, seed=0)
    sizes = m.cell_sizes()
    core, outer = sizes[:ni * nj], sizes[ni * nj:]
    # quads; the outermost core ring also carries the nodes where the
    # polygonal region meets it
    assert (core[:ni * (nj - 1)] == 4).all() and core[ni * (nj - 1):].min() >= 4
    assert outer.size > 0 and outer.min() >= 3 and outer.max() <= 9
    assert ((outer >= 4) & (outer <= 9)).mean() > 0.999
    assert (outer >= 5).mean() > 0.5  # polygons, not quads
    # farfield polygon: vertices on (and just inside) the 20-chord circle
    r, _, far = _wall_and_far(m)
    assert r[far].max() <= 20.0 + 1e-12 and r[far].min() >= 20.0 * (1 - 1e-4)


def test_naca4412_hybrid_structure():
    ni, layers = 256, 40
    m = meshgen.naca_hybrid(ni, layers, tri_rows=120)
    sizes = m.cell_sizes()
    assert (sizes == 4).sum() == ni * layers and (sizes == 3).sum() == m.n_cells - ni * layers
    r, wall, far = _wall_and_far(m)
    np.testing.assert_allclose(r[far], 30.0, rtol=1e-12)
    # cambered section: the wall is not symmetric about y = 0
    assert abs(m.nodes[wall][:, 1].max() + m.nodes[wall][:, 1].min()) > 0.02
    sp = _first_spacing(m, wall)
    assert abs(np.median(sp) - 4.5e-6) < 0.1 * 4.5e-6
    # y+ of the first cell at Re 6e6 from the flat-plate skin friction
    # Cf = 0.026 Re^(-1/7): about 1
    re = 6e6
    yplus = np.median(sp) * re * np.sqrt(0.5 * 0.026 * re ** (-1.0 / 7.0))
    assert 0.7 < yplus < 1.4
    # a valid mesh: across every face the neighbour's centroid lies on the
    # far side (positive face-normal distance, which the RANS time step
    # divides by), i.e. no two triangles overlap
    assert _min_normal_distance_cos(m) > 0.0


def _min_normal_distance_cos(poly):
    from finitevolume_gb300 import solvers as S
    ex = S.Mesh(poly, reorder="none").export()
    fi, fd, cd = ex["faces_i32"], ex["faces_f64"], ex["cells_f64"]
    L, R = fi[:, 2], fi[:, 3]
    xr = np.where(R >= 0, cd[np.maximum(R, 0), 1], fd[:, 3])
    yr = np.where(R >= 0, cd[np.maximum(R, 0), 2], fd[:, 4])
    dx, dy = xr - cd[L, 1], yr - cd[L, 2]
    return float(((fd[:, 0] * dx + fd[:, 1] * dy) / np.hypot(dx, dy)).min())


def test_batch_family_ranges():
    cases = meshgen.batch_cases(256, seed=0)
    assert len(cases) == 256
    camber = np.array([c["shape"][0] for c in cases])
    thick = np.array([c["shape"][2] for c in cases])
    cells = np.array([c["ni"] * c["nj"] for c in cases])
    mach = np.array([c["mach"] for c in cases])
    aoa = np.array([c["aoa_deg"] for c in cases])
    assert camber.min() >= 0.0 and camber.max() <= 0.06 and camber.max() - camber.min() > 0.05
    assert thick.min() >= 0.08 and thick.max() <= 0.18 and thick.max() - thick.min() > 0.08
    assert mach.min() >= 0.3 and mach.max() <= 0.85 and mach.max() - mach.min() > 0.45
    assert aoa.min() >= -4.0 and aoa.max() <= 8.0 and aoa.max() - aoa.min() > 10.0
    # log-uniform cell counts over 4k..64k (within the rounding of nj)
    assert cells.min() >= 0.9 * 4096 and cells.max() <= 1.1 * 65536
    lc = np.log(cells)
    assert abs(np.median(lc) - 0.5 * (np.log(4096) + np.log(65536))) < 0.3
    assert [c["ni"] for c in cases] == [2 * c["nj"] for c in cases]
    # seeded: the same family every time
    again = meshgen.batch_cases(256, seed=0)
    assert all(a == b for a, b in zip(cases, again))


def test_surface_displacement_directions():
    """The shape-gradient check's directions: seeded white noise on the
    wall nodes smoothed by a Gaussian over 20 nodes, along the unit wall
    normal, zero elsewhere, scaled to a maximum of 1."""
    poly = meshgen.naca_ogrid(128, 32)
    dirs = meshgen.wall_normal_directions(poly, 16, seed=0, width=20)
    assert len(dirs) == 16
    _, wall, _ = _wall_and_far(poly)
    off_wall = np.setdiff1d(np.arange(poly.nodes.shape[0]), wall)
    for d in dirs:
        assert d.shape == poly.nodes.shape
        assert not d[off_wall].any()
        mag = np.hypot(d[wall, 0], d[wall, 1])
        np.testing.assert_allclose(mag.max(), 1.0, rtol=1e-12)
    # normal to the wall: orthogonal to the local tangent (central difference
    # along the wall loop)
    e = poly.bedges[poly.bpatch == list(poly.patch_names).index("airfoil")]
    nxt = {int(a): int(b) for a, b in e}
    order = [int(e[0, 0])]
    while nxt[order[-1]] != order[0]:
        order.append(nxt[order[-1]])
    P = poly.nodes[order]
    tang = np.roll(P, -1, axis=0) - np.roll(P, 1, axis=0)
    for d in dirs:
        dd = d[order]
        assert np.abs(np.sum(dd * tang, axis=1)).max() <= 1e-12 * np.abs(tang).max()
    # smooth: neighbouring wall nodes move alike (white noise would not)
    a = np.array([np.sum(d[order] * np.stack([tang[:, 1], -tang[:, 0]], 1), axis=1) for d in dirs])
    a /= np.abs(a).max(axis=1, keepdims=True)
    jumps = np.abs(np.diff(a, axis=1)).max()
    assert jumps < 0.3
    # seeded
    again = meshgen.wall_normal_directions(poly, 16, seed=0, width=20)
    assert all(np.array_equal(x, y) for x, y in zip(dirs, again))
    assert not np.array_equal(dirs[0], meshgen.wall_normal_directions(poly, 1, seed=1, width=20)[0])
