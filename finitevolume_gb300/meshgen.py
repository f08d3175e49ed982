"""Seeded synthetic mesh generators for the benchmark and parity cases.

All generators return a :class:`~finitevolume_gb300.fvmesh.PolyMesh` with
counter-clockwise cells and tagged boundary edges, ready for
``write_fvmesh`` (reference side) and ``Mesh.from_polymesh`` (GPU side).

* :func:`naca_ogrid`     NACA 4-digit O-grid (closed trailing edge, geometric
                         wall-normal stretching, circular farfield)
* :func:`naca_mixed`     O-grid core + a Lloyd-relaxed polygonal outer region
                         (dual of a Delaunay triangulation; cells of 3-11
                         sides, more than 99.9% of them 4-9)
* :func:`sod_strip`      randomly perturbed triangle strip (shock tube)
* :func:`wavy_quads`     non-affine ("wavy") structured quads, for gradient
                         exactness checks
* :func:`cartesian`      plain structured quads

NACA sections come from the public 4-digit formula (thickness polynomial with
the -0.1036 x^4 coefficient that closes the trailing edge).
"""
from __future__ import annotations

import math
from typing import Tuple

import numpy as np

from .fvmesh import PolyMesh, from_cells, signed_areas


# --------------------------------------------------------------------------
# NACA 4-digit geometry
# --------------------------------------------------------------------------
def naca4(code: str, x: np.ndarray) -> Tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
    """Upper and lower surface coordinates at chord stations ``x`` in [0, 1]."""
    m = int(code[0]) / 100.0
    p = int(code[1]) / 10.0
    t = int(code[2:]) / 100.0
    return naca4_params(m, p, t, x)


def naca4_params(m: float, p: float, t: float, x: np.ndarray):
    yt = 5.0 * t * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x**2 + 0.2843 * x**3 - 0.1036 * x**4)
    if m > 0.0 and p > 0.0:
        yc = np.where(x < p, m / p**2 * (2 * p * x - x**2), m / (1 - p)**2 * ((1 - 2 * p) + 2 * p * x - x**2))
        dyc = np.where(x < p, 2 * m / p**2 * (p - x), 2 * m / (1 - p)**2 * (p - x))
    else:
        yc = np.zeros_like(x)
        dyc = np.zeros_like(x)
    th = np.arctan(dyc)
    xu, yu = x - yt * np.sin(th), yc + yt * np.cos(th)
    xl, yl = x + yt * np.sin(th), yc - yt * np.cos(th)
    return xu, yu, xl, yl


def airfoil_loop(ni: int, m: float = 0.0, p: float = 0.0, t: float = 0.12) -> np.ndarray:
    """``ni`` surface points, TE -> upper -> LE -> lower, counter-clockwise.

    Cosine clustering in chord; point 0 is the (closed) trailing edge.
    """
    if ni % 2:
        raise ValueError("ni must be even")
    h = ni // 2
    s_up = np.linspace(1.0, 0.0, h + 1)          # TE .. LE inclusive
    s_lo = np.linspace(0.0, 1.0, h + 1)[1:-1]    # LE .. TE exclusive
    xu_c = 0.5 * (1.0 - np.cos(np.pi * s_up))
    xl_c = 0.5 * (1.0 - np.cos(np.pi * s_lo))
    xu, yu, _, _ = naca4_params(m, p, t, xu_c)
    _, _, xl, yl = naca4_params(m, p, t, xl_c)
    pts = np.concatenate([np.stack([xu, yu], 1), np.stack([xl, yl], 1)], 0)
    pts[0] = (1.0, 0.0)
    pts[h] = (0.0, 0.0)
    return pts


def _stretch(n: int, first: float, total: float) -> np.ndarray:
    """Cumulative distances 0..total over n geometric intervals, first = ``first``."""
    if first * n >= total:
        return np.linspace(0.0, total, n + 1)
    lo, hi = 1.0 + 1e-12, 2.0
    for _ in range(200):
        g = 0.5 * (lo + hi)
        s = first * (g**n - 1.0) / (g - 1.0)
        lo, hi = (g, hi) if s < total else (lo, g)
    g = 0.5 * (lo + hi)
    d = first * (g ** np.arange(n + 1) - 1.0) / (g - 1.0)
    return d * (total / d[-1])


def _ogrid_nodes(ni: int, nj: int, first: float, r_out: float, center=(0.5, 0.0), m=0.0, p=0.0, t=0.12):
    """O-grid node array [nj+1, ni, 2]; ring nj lies on the circle r_out."""
    s = airfoil_loop(ni, m, p, t)
    c = np.asarray(center)
    # Outward unit normals (right of the CCW traversal), central differences.
    tang = np.roll(s, -1, axis=0) - np.roll(s, 1, axis=0)
    nrm = np.stack([tang[:, 1], -tang[:, 0]], 1)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    theta = 2.0 * np.pi * np.arange(ni) / ni
    circ = c + r_out * np.stack([np.cos(theta), np.sin(theta)], 1)
    dist = np.linalg.norm(circ - s, axis=1)
    d = _stretch(nj, first, float(dist.mean()))
    f = d / d[-1]
    w = f ** 0.5
    nodes = np.empty((nj + 1, ni, 2))
    for j in range(nj + 1):
        pn = s + (d[j] * dist / d[-1])[:, None] * nrm
        ps = s + f[j] * (circ - s)
        nodes[j] = (1.0 - w[j]) * pn + w[j] * ps
    nodes[nj] = circ
    return nodes


def naca_ogrid(ni: int = 256, nj: int = 128, first: float = 1e-3, r_far: float = 20.0,
               code: str = "0012", shape=None) -> PolyMesh:
    """NACA 4-digit O-grid: ``ni`` cells around, ``nj`` radially.

    ``shape`` = (max camber, camber position, thickness) as chord fractions
    overrides the 4-digit ``code`` (non-integer sections).  Patches:
    ``airfoil`` (the wall) and ``farfield`` (circle of radius ``r_far``
    chords about mid-chord).
    """
    if shape is not None:
        m, p, t = (float(x) for x in shape)
    else:
        m, p, t = int(code[0]) / 100.0, int(code[1]) / 10.0, int(code[2:]) / 100.0
    nodes3 = _ogrid_nodes(ni, nj, first, r_far, m=m, p=p, t=t)
    nodes = nodes3.reshape(-1, 2)
    jj, ii = np.meshgrid(np.arange(nj), np.arange(ni), indexing="ij")
    a = jj * ni + ii
    b = jj * ni + (ii + 1) % ni
    cells = np.stack([a, b, b + ni, a + ni], -1).reshape(-1, 4)
    wall = np.stack([np.arange(ni), (np.arange(ni) + 1) % ni], 1)
    far = nj * ni + wall
    mesh = from_cells(nodes, cells, np.concatenate([wall, far]),
                      np.r_[np.zeros(ni, np.int32), np.ones(ni, np.int32)], ["airfoil", "farfield"])
    _orient(mesh)
    return mesh


def _orient(mesh: PolyMesh) -> None:
    """Reverse the vertex order of any clockwise cell in place."""
    a = signed_areas(mesh)
    bad = np.nonzero(a < 0.0)[0]
    for c in bad:
        lo, hi = mesh.cell_off[c], mesh.cell_off[c + 1]
        mesh.cell_nodes[lo:hi] = mesh.cell_nodes[lo:hi][::-1]


# --------------------------------------------------------------------------
# Mixed mesh: O-grid core + Lloyd-relaxed polygonal outer region
# --------------------------------------------------------------------------
def _circumcenters(p: np.ndarray, tri: np.ndarray) -> np.ndarray:
    a, b, c = p[tri[:, 0]], p[tri[:, 1]], p[tri[:, 2]]
    ax, ay = a[:, 0], a[:, 1]
    bx, by = b[:, 0] - ax, b[:, 1] - ay
    cx, cy = c[:, 0] - ax, c[:, 1] - ay
    d = 2.0 * (bx * cy - by * cx)
    b2, c2 = bx * bx + by * by, cx * cx + cy * cy
    ux = (cy * b2 - by * c2) / d
    uy = (bx * c2 - cx * b2) / d
    return np.stack([ax + ux, ay + uy], 1)


def _fans(tri: np.ndarray, pts: np.ndarray, vert_xy: np.ndarray, n_vert: int):
    """Group (vertex, triangle) incidences by vertex, sorted by angle.

    Returns (order, starts): ``order`` lists triangle ids, grouped per vertex
    0..n_vert-1 and sorted counter-clockwise by the angle of ``pts[t]`` about
    ``vert_xy[v]``; ``starts[v]:starts[v+1]`` is vertex v's group.
    """
    v = tri.reshape(-1)
    t = np.repeat(np.arange(tri.shape[0]), 3)
    keep = v < n_vert
    v, t = v[keep], t[keep]
    d = pts[t] - vert_xy[v]
    ang = np.arctan2(d[:, 1], d[:, 0])
    o = np.lexsort((ang, v))
    counts = np.bincount(v, minlength=n_vert)
    starts = np.zeros(n_vert + 1, dtype=np.int64)
    np.cumsum(counts, out=starts[1:])
    return t[o], starts, v[o]


def _poly_centroids(poly_xy: np.ndarray, starts: np.ndarray) -> np.ndarray:
    """Centroids of closed polygons given as grouped vertex lists."""
    n = starts.size - 1
    sizes = np.diff(starts)
    idx = np.arange(poly_xy.shape[0])
    nxt = idx + 1
    nxt[starts[1:] - 1] = starts[:-1]
    p0, p1 = poly_xy, poly_xy[nxt]
    cr = p0[:, 0] * p1[:, 1] - p1[:, 0] * p0[:, 1]
    g = np.repeat(np.arange(n), sizes)
    a = np.bincount(g, cr, n) * 0.5
    cx = np.bincount(g, (p0[:, 0] + p1[:, 0]) * cr, n) / (6.0 * a)
    cy = np.bincount(g, (p0[:, 1] + p1[:, 1]) * cr, n) / (6.0 * a)
    return np.stack([cx, cy], 1)


def _periodic_delaunay(fixed: np.ndarray, free: np.ndarray, period: float, band: float):
    """Delaunay of points periodic in y; returns (triangles over base ids, n_base).

    Base ids: free points first, then fixed points.  Triangles are kept once
    (centroid y in [0, period)).
    """
    from scipy.spatial import Delaunay

    base = np.concatenate([free, fixed], 0)
    nb = base.shape[0]
    lo = base[:, 1] < band
    hi = base[:, 1] >= period - band
    ext = np.concatenate([base, base[lo] + [0.0, period], base[hi] - [0.0, period]], 0)
    ids = np.concatenate([np.arange(nb), np.nonzero(lo)[0], np.nonzero(hi)[0]])
    tri = Delaunay(ext).simplices
    cy = ext[tri, 1].mean(1)
    tri = tri[(cy >= 0.0) & (cy < period)]
    return tri, ids, ext


def naca_mixed(ni: int = 1024, nj: int = 512, first: float = 1e-3, r_core: float = 2.0,
               r_far: float = 20.0, code: str = "0012", lloyd_iters: int = 4, seed: int = 0) -> PolyMesh:
    """NACA O-grid core of ni x nj quads, surrounded by a polygonal region.

    The outer region (r_core < r < r_far about mid-chord) is built in
    log-polar coordinates (xi = ln r, eta = angle), where uniform point
    density gives cells whose size grows in proportion to r.  Seeded uniform
    random points are relaxed by ``lloyd_iters`` Lloyd iterations
    (Voronoi-centroid moves, periodic in eta), then triangulated; each point
    becomes one polygonal cell whose vertices are the centroids of its
    Delaunay triangles (the centroid dual: always a simple, star-shaped
    polygon; after relaxation more than 99.9% of them have 4-9 sides).  The
    few with 10 or more sides are split in two along a chord between two of
    their vertices, so every outer cell has 3-9 sides.  The core's outer
    ring nodes are
    the dual's inner boundary vertices: their cells close on the ring edge
    midpoints, which also become the fifth vertex of the core's outermost
    quads, so the two regions share faces exactly.

    Patches: ``airfoil`` (wall), ``farfield``.
    """
    rng = np.random.default_rng(seed)
    m, p, t = int(code[0]) / 100.0, int(code[1]) / 10.0, int(code[2:]) / 100.0
    center = np.array([0.5, 0.0])
    core = _ogrid_nodes(ni, nj, first, r_core, center=center, m=m, p=p, t=t)

    two_pi = 2.0 * np.pi
    dlt = two_pi / ni
    xi0, xi1 = math.log(r_core), math.log(r_far)
    n_far = ni
    eta_in = two_pi * np.arange(ni) / ni
    eta_out = two_pi * (np.arange(n_far) + 0.5) / n_far
    row = dlt * math.sqrt(3.0) / 2.0
    ring_in = np.stack([np.full(ni, xi0), eta_in], 1)
    ring_out = np.stack([np.full(n_far, xi1), eta_out], 1)
    ghost_in = np.stack([np.full(ni, xi0 - row), eta_in + 0.5 * dlt], 1) % [np.inf, two_pi]
    ghost_out = np.stack([np.full(n_far, xi1 + row), eta_out + 0.5 * dlt], 1) % [np.inf, two_pi]
    fixed = np.concatenate([ring_in, ring_out, ghost_in, ghost_out], 0)

    area = (xi1 - xi0 - 2 * 0.5 * dlt) * two_pi
    n_free = int(round(area / (dlt * dlt * math.sqrt(3.0) / 2.0)))
    free = np.stack([rng.uniform(xi0 + 0.5 * dlt, xi1 - 0.5 * dlt, n_free),
                     rng.uniform(0.0, two_pi, n_free)], 1)
    band = 12.0 * dlt
    for _ in range(lloyd_iters):
        tri, ids, ext = _periodic_delaunay(fixed, free, two_pi, band)
        cc = _circumcenters(ext, tri)
        vid = ids[tri]
        order, starts, _ = _fans(vid, cc, np.concatenate([free, fixed]), n_free)
        cen = _poly_centroids(cc[order], starts)
        # Clamp so the free points stay strictly inside the band.
        cen[:, 0] = np.clip(cen[:, 0], xi0 + 0.3 * dlt, xi1 - 0.3 * dlt)
        free = np.stack([cen[:, 0], cen[:, 1] % two_pi], 1)

    tri, ids, ext = _periodic_delaunay(fixed, free, two_pi, band)
    vid = ids[tri]
    n_keep = n_free + ni + n_far          # free, inner ring, outer ring (no ghosts)
    tri_ok = (vid < n_keep).all(1)
    vid = vid[tri_ok]
    base = np.concatenate([free, fixed[:ni + n_far]], 0)
    phys = center + np.exp(base[:, :1]) * np.stack([np.cos(base[:, 1]), np.sin(base[:, 1])], 1)
    # The inner ring must coincide with the core's outer ring nodes exactly.
    phys[n_free:n_free + ni] = core[nj]
    # Orient every triangle CCW in physical space.
    a, b, c = phys[vid[:, 0]], phys[vid[:, 1]], phys[vid[:, 2]]
    cr = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    vid[cr < 0] = vid[cr < 0][:, ::-1]
    tcen = phys[vid].mean(1)
    n_tri = vid.shape[0]

    # ---- node numbering of the final mesh --------------------------------
    n_core = (nj + 1) * ni
    k_in = np.arange(ni)
    off_mid_in = n_core
    off_tri = off_mid_in + ni
    off_out = off_tri + n_tri
    off_mid_out = off_out + n_far
    mid_in = 0.5 * (core[nj][k_in] + core[nj][(k_in + 1) % ni])
    out_xy = phys[n_free + ni:n_keep]
    mid_out = 0.5 * (out_xy + np.roll(out_xy, -1, axis=0))
    nodes = np.concatenate([core.reshape(-1, 2), mid_in, tcen, out_xy, mid_out], 0)

    def node_of_base(v):
        v = np.asarray(v)
        return np.where(v < n_free, -1, np.where(v < n_free + ni, nj * ni + (v - n_free), off_out + (v - n_free - ni)))

    cells = []
    # Core quads j < nj-1 and pentagons at j = nj-1 (outer edge split at the midpoint).
    for j in range(nj):
        i = np.arange(ni)
        a0 = j * ni + i
        b0 = j * ni + (i + 1) % ni
        if j < nj - 1:
            cells.extend(np.stack([a0, b0, b0 + ni, a0 + ni], 1).tolist())
        else:
            cells.extend(np.stack([a0, b0, b0 + ni, off_mid_in + i, a0 + ni], 1).tolist())
    core_cells = len(cells)

    order, starts, _ = _fans(vid, tcen, phys, n_keep)
    tri_node = off_tri + order
    # Interior points: closed fans.
    for v in range(n_free):
        cells.append(tri_node[starts[v]:starts[v + 1]].tolist())
    # Ring points: open fans closed by the ring vertex and two edge midpoints.
    for k in range(ni):
        v = n_free + k
        w = phys[v]
        fan_t = order[starts[v]:starts[v + 1]]
        outward = w - center
        outward /= np.linalg.norm(outward)
        tang = np.array([-outward[1], outward[0]])        # CCW tangent (toward ring k+1)
        d = tcen[fan_t] - w
        ang = np.arctan2(d @ outward, d @ tang)           # 0 at +tangent, pi at -tangent
        fan = off_tri + fan_t[np.argsort(ang)]
        cells.append([nj * ni + k, off_mid_in + k] + fan.tolist() + [off_mid_in + (k - 1) % ni])
    for k in range(n_far):
        v = n_free + ni + k
        w = phys[v]
        fan_t = order[starts[v]:starts[v + 1]]
        inward = center - w
        inward /= np.linalg.norm(inward)
        tang = np.array([-inward[1], inward[0]])          # CW along the ring (toward k-1)
        d = tcen[fan_t] - w
        ang = np.arctan2(d @ inward, d @ tang)
        fan = off_tri + fan_t[np.argsort(ang)]
        cells.append([off_out + k, off_mid_out + (k - 1) % n_far] + fan.tolist() + [off_mid_out + k])

    cells = _split_polygons(nodes, cells, max_sides=9)

    wall = np.stack([np.arange(ni), (np.arange(ni) + 1) % ni], 1)
    kk = np.arange(n_far)
    far = np.concatenate([np.stack([off_out + kk, off_mid_out + kk], 1),
                          np.stack([off_mid_out + kk, off_out + (kk + 1) % n_far], 1)])
    mesh = from_cells(nodes, cells, np.concatenate([wall, far]),
                      np.r_[np.zeros(ni, np.int32), np.ones(far.shape[0], np.int32)], ["airfoil", "farfield"])
    _orient(mesh)
    mesh.validate_ccw()
    return mesh


def _split_polygons(nodes, cells, max_sides: int = 9):
    """Split every cell with more than ``max_sides`` vertices in two along a
    chord between two of its vertices about half-way round (n vertices give
    halves of n//2 + 1 and n - n//2 + 1).  No vertex is added, so the
    neighbouring cells keep their faces.  Of the n candidate chords the one
    whose halves are both convex and have the largest smaller area is
    taken (failing convexity: the largest smaller signed area).  Cells keep
    their vertex orientation."""
    def signed_area(p):
        x, y = p[:, 0], p[:, 1]
        return 0.5 * float(np.sum(x * np.roll(y, -1) - np.roll(x, -1) * y))

    def convex(p, sgn):
        d1 = np.roll(p, -1, axis=0) - p
        d2 = np.roll(d1, -1, axis=0)
        return bool((sgn * (d1[:, 0] * d2[:, 1] - d1[:, 1] * d2[:, 0]) > 0).all())

    out = []
    for c in cells:
        n = len(c)
        if n <= max_sides:
            out.append(c)
            continue
        pts = nodes[np.asarray(c)]
        sgn = 1.0 if signed_area(pts) > 0 else -1.0
        best, best_key = None, None
        for i in range(n):
            j = (i + n // 2) % n
            a = [c[(i + k) % n] for k in range((j - i) % n + 1)]
            b = [c[(j + k) % n] for k in range((i - j) % n + 1)]
            pa, pb = nodes[np.asarray(a)], nodes[np.asarray(b)]
            key = (convex(pa, sgn) and convex(pb, sgn), min(sgn * signed_area(pa), sgn * signed_area(pb)))
            if best_key is None or key > best_key:
                best, best_key = (a, b), key
        out.extend(_split_polygons(nodes, list(best), max_sides))
    return out


def naca_hybrid(ni: int = 1024, n_layers: int = 40, first: float = 4.5e-6, growth: float = 1.15,
                r_far: float = 30.0, code: str = "4412", tri_rows: int = 955, jitter: float = 0.3,
                seed: int = 0) -> PolyMesh:
    """Hybrid RANS mesh about a NACA 4-digit section.

    ``n_layers`` wall-clustered quad layers (first spacing ``first`` chords,
    geometric ``growth``) along the smoothed surface normals, then seeded
    random triangles out to a farfield circle of radius ``r_far`` about
    mid-chord.  The triangle nodes are the nodes of an auxiliary O-grid of
    ``tri_rows`` rows moved by seeded uniform offsets of up to ``jitter``
    cells (in its index space, mapped back bilinearly); the triangles are
    their physical-space Delaunay triangulation together with the
    outermost quad ring and the farfield ring, which fills the annulus
    between them and shares their nodes.  The
    default (1024 around, 40 layers, 955 rows) has 1.99M cells; the first
    spacing is y+ ~ 1 at Re_c = 6e6 by the flat-plate estimate.

    Patches: ``airfoil`` (wall), ``farfield``.
    """
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    m, p, t = int(code[0]) / 100.0, int(code[1]) / 10.0, int(code[2:]) / 100.0
    s0 = airfoil_loop(ni, m, p, t)
    tang = np.roll(s0, -1, axis=0) - np.roll(s0, 1, axis=0)
    nrm = np.stack([tang[:, 1], -tang[:, 0]], 1)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    d = first * (growth ** np.arange(n_layers + 1) - 1.0) / (growth - 1.0)
    quad = s0[None, :, :] + d[:, None, None] * nrm[None, :, :]          # [L+1, ni, 2]
    # auxiliary O-grid from the outermost layer to the farfield circle
    inner = quad[-1]
    center = np.array([0.5, 0.0])
    theta = 2.0 * np.pi * np.arange(ni) / ni
    circ = center + r_far * np.stack([np.cos(theta), np.sin(theta)], 1)
    dist = np.linalg.norm(circ - inner, axis=1)
    k_first = (d[-1] - d[-2]) * growth
    e = _stretch(tri_rows, k_first, float(dist.mean()))
    f = e / e[-1]
    w = f ** 0.5
    aux = np.empty((tri_rows + 1, ni, 2))
    for k in range(tri_rows + 1):
        pn = inner + (e[k] * dist / e[-1])[:, None] * nrm
        ps = inner + f[k] * (circ - inner)
        aux[k] = (1.0 - w[k]) * pn + w[k] * ps
    aux[0] = inner
    aux[-1] = circ
    # jittered interior points in index space (rows 1..K-1, periodic in i),
    # mapped bilinearly to physical space
    K = tri_rows
    ii, kk = np.meshgrid(np.arange(ni, dtype=np.float64), np.arange(1, K, dtype=np.float64))
    kq = kk.ravel() + rng.uniform(-jitter, jitter, kk.size)
    iq = (ii.ravel() + rng.uniform(-jitter, jitter, ii.size)) % ni
    k0 = np.clip(np.floor(kq).astype(np.int64), 0, K - 1)
    i0 = np.floor(iq).astype(np.int64) % ni
    a_, b_ = kq - k0, iq - np.floor(iq)
    i1 = (i0 + 1) % ni
    xy = ((1 - a_)[:, None] * ((1 - b_)[:, None] * aux[k0, i0] + b_[:, None] * aux[k0, i1])
          + a_[:, None] * ((1 - b_)[:, None] * aux[k0 + 1, i0] + b_[:, None] * aux[k0 + 1, i1]))
    # Free points inside the diametral circle of a ring edge are dropped,
    # so that every ring edge is a Gabriel edge and hence an edge of the
    # Delaunay triangulation below.
    from scipy.spatial import cKDTree
    tree = cKDTree(xy)
    drop = set()
    for ring in (inner, circ):
        a, b = ring, np.roll(ring, -1, axis=0)
        mid, rad = 0.5 * (a + b), 0.5 * np.linalg.norm(b - a, axis=1)
        for j, hits in enumerate(tree.query_ball_point(mid, rad * (1.0 + 1e-9))):
            drop.update(hits)
    if drop:
        xy = np.delete(xy, np.fromiter(sorted(drop), np.int64), axis=0)
    nf = xy.shape[0]
    # Delaunay of those points with both rings, in physical space (a
    # triangulation taken in index space and mapped puts thin triangles on
    # the wrong side of their neighbours where the aux grid is strongly
    # anisotropic, behind the trailing edge): two triangles sharing an edge
    # then lie on opposite sides of it, so every face-normal distance
    # between centroids is positive.  Triangles with all three vertices on
    # the inner ring and their centroid inside it fill the airfoil and the
    # quad layers and are dropped; every ring edge must be a triangle edge.
    pts = np.concatenate([xy, inner, circ], 0)
    tri = Delaunay(pts).simplices
    on_inner = np.zeros(pts.shape[0], bool)
    on_inner[nf:nf + ni] = True
    cand = np.nonzero(on_inner[tri].all(1))[0]
    cen = pts[tri[cand]].mean(1)
    x, y = cen[:, 0][:, None], cen[:, 1][:, None]
    x1, y1 = inner[:, 0][None], inner[:, 1][None]
    x2, y2 = np.roll(inner, -1, 0)[:, 0][None], np.roll(inner, -1, 0)[:, 1][None]
    cross = ((y1 > y) != (y2 > y)) & (x < (x2 - x1) * (y - y1) / np.where(y2 != y1, y2 - y1, 1.0) + x1)
    keep = np.ones(tri.shape[0], bool)
    keep[cand[cross.sum(1) % 2 == 1]] = False
    tri = tri[keep]
    # node numbering: quad layers (rows 0..L, ring L = aux ring 0), then the
    # free triangle nodes, then the farfield ring
    L = n_layers
    n_quad_nodes = (L + 1) * ni
    nodes = np.concatenate([quad.reshape(-1, 2), xy, circ], 0)
    pmap = np.concatenate([n_quad_nodes + np.arange(nf), L * ni + np.arange(ni), n_quad_nodes + nf + np.arange(ni)])
    tris = pmap[tri]
    edges = np.sort(np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]], 0), axis=1)
    edge_keys = set((edges[:, 0] * nodes.shape[0] + edges[:, 1]).tolist())
    for ring0 in (L * ni, n_quad_nodes + nf):
        a = ring0 + np.arange(ni)
        b = ring0 + (np.arange(ni) + 1) % ni
        keys = np.minimum(a, b) * nodes.shape[0] + np.maximum(a, b)
        if not all(int(k) in edge_keys for k in keys):
            raise RuntimeError("naca_hybrid: a ring edge is missing from the triangulation")
    P = nodes[tris]
    area2 = (P[:, 1, 0] - P[:, 0, 0]) * (P[:, 2, 1] - P[:, 0, 1]) - (P[:, 2, 0] - P[:, 0, 0]) * (P[:, 1, 1] - P[:, 0, 1])
    tris[area2 < 0] = tris[area2 < 0][:, ::-1]
    jj, ii2 = np.meshgrid(np.arange(L), np.arange(ni), indexing="ij")
    a0 = jj * ni + ii2
    b0 = jj * ni + (ii2 + 1) % ni
    quads = np.stack([a0, b0, b0 + ni, a0 + ni], -1).reshape(-1, 4)
    cells = [list(q) for q in quads] + [list(t) for t in tris]
    wall = np.stack([np.arange(ni), (np.arange(ni) + 1) % ni], 1)
    far = n_quad_nodes + nf + np.stack([np.arange(ni), (np.arange(ni) + 1) % ni], 1)
    mesh = from_cells(nodes, cells, np.concatenate([wall, far]),
                      np.r_[np.zeros(ni, np.int32), np.ones(ni, np.int32)], ["airfoil", "farfield"])
    _orient(mesh)
    return mesh


def wall_normal_directions(poly: PolyMesh, n_dirs: int, seed: int = 0, width: int = 20, patch: int = 0):
    """Seeded surface-normal displacement fields of one closed wall loop
    (boundary patch ``patch``): white noise on the wall nodes smoothed by a
    periodic Gaussian over ``width`` nodes (sigma width/3), times the unit
    node normal; each field [n_nodes, 2] scaled to a maximum of 1 and zero
    off the wall."""
    e = poly.bedges[poly.bpatch == patch]
    nxt = {int(a): int(b) for a, b in e}
    order = [int(e[0, 0])]
    while nxt[order[-1]] != order[0]:
        order.append(nxt[order[-1]])
    order = np.array(order)
    P = poly.nodes[order]
    t = np.roll(P, -1, axis=0) - np.roll(P, 1, axis=0)
    nrm = np.stack([t[:, 1], -t[:, 0]], 1)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    rng = np.random.default_rng(seed)
    k = np.arange(-width, width + 1)
    ker = np.exp(-0.5 * (k / (width / 3.0)) ** 2)
    out = []
    for _ in range(n_dirs):
        w = rng.standard_normal(len(order))
        a = sum(ker[j] * np.roll(w, k[j]) for j in range(len(k)))
        a /= np.abs(a).max()
        d = np.zeros_like(poly.nodes)
        d[order] = a[:, None] * nrm
        out.append(d)
    return out


CACHE_VERSION = 4  # 2: naca_mixed splits cells of more than 9 sides; 3: naca_hybrid triangulated in physical space; 4: without ring-encroaching points


def cached(name: str, **kw) -> PolyMesh:
    """Generate ``name(**kw)`` once and keep it as .npz in a cache folder.

    The folder is ``$FV_MESH_CACHE`` or ``~/.cache/finitevolume_gb300``; the
    key is the generator name, its keyword arguments and ``CACHE_VERSION``
    (raised whenever a generator's output changes).
    """
    import hashlib
    import json
    import os

    from .fvmesh import PolyMesh as _PM

    root = os.environ.get("FV_MESH_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "finitevolume_gb300"))
    key = hashlib.sha256(json.dumps([name, sorted(kw.items()), CACHE_VERSION], default=str).encode()).hexdigest()[:16]
    path = os.path.join(root, f"{name}_{key}.npz")
    if os.path.exists(path):
        z = np.load(path, allow_pickle=False)
        return _PM(z["nodes"], z["cell_off"], z["cell_nodes"], z["bedges"], z["bpatch"],
                   [str(x) for x in z["patch_names"]])
    m = globals()[name](**kw)
    os.makedirs(root, exist_ok=True)
    tmp = path + f".{os.getpid()}.tmp.npz"
    np.savez(tmp, nodes=m.nodes, cell_off=m.cell_off, cell_nodes=m.cell_nodes, bedges=m.bedges, bpatch=m.bpatch,
             patch_names=np.array(m.patch_names))
    os.replace(tmp, path)
    return m


# --------------------------------------------------------------------------
# Simple test meshes
# --------------------------------------------------------------------------
def cartesian(nx: int, ny: int, lx: float = 1.0, ly: float = 1.0) -> PolyMesh:
    """Structured quads on [0,lx]x[0,ly]; patches bottom,right,top,left."""
    x = np.linspace(0.0, lx, nx + 1)
    y = np.linspace(0.0, ly, ny + 1)
    X, Y = np.meshgrid(x, y)
    return _structured(np.stack([X.ravel(), Y.ravel()], 1), nx, ny)


def wavy_quads(n: int = 8, amp: float = 0.04) -> PolyMesh:
    """Unit-square quads with a smooth non-affine interior perturbation."""
    x = np.linspace(0.0, 1.0, n + 1)
    X, Y = np.meshgrid(x, x)
    dx = amp * np.sin(2 * np.pi * Y) * np.sin(np.pi * X)
    dy = amp * np.sin(2 * np.pi * X) * np.sin(np.pi * Y)
    return _structured(np.stack([(X + dx).ravel(), (Y + dy).ravel()], 1), n, n)


def _structured(nodes: np.ndarray, nx: int, ny: int) -> PolyMesh:
    jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    a = jj * (nx + 1) + ii
    cells = np.stack([a, a + 1, a + nx + 2, a + nx + 1], -1).reshape(-1, 4)
    i = np.arange(nx)
    j = np.arange(ny)
    bottom = np.stack([i, i + 1], 1)
    top = np.stack([ny * (nx + 1) + i + 1, ny * (nx + 1) + i], 1)
    left = np.stack([(j + 1) * (nx + 1), j * (nx + 1)], 1)
    right = np.stack([j * (nx + 1) + nx, (j + 1) * (nx + 1) + nx], 1)
    be = np.concatenate([bottom, right, top, left])
    bp = np.repeat(np.arange(4, dtype=np.int32), [nx, ny, nx, ny])
    return from_cells(nodes, cells, be, bp, ["bottom", "right", "top", "left"])


def sod_strip(nx: int, ny: int, length: float = 1.0, height: float = None, jitter: float = 0.2,
              seed: int = 0) -> PolyMesh:
    """Randomly perturbed triangle strip on [0,length] x [0,height].

    ``nx * ny`` rectangles, each split along a randomly chosen diagonal;
    interior nodes moved by up to ``jitter`` of the local spacing.  Patches:
    bottom, right, top, left.  2*nx*ny triangles.
    """
    rng = np.random.default_rng(seed)
    if height is None:
        height = length * ny / nx
    x = np.linspace(0.0, length, nx + 1)
    y = np.linspace(0.0, height, ny + 1)
    X, Y = np.meshgrid(x, y)
    hx, hy = length / nx, height / ny
    inner = np.zeros_like(X, dtype=bool)
    inner[1:-1, 1:-1] = True
    X = X + np.where(inner, rng.uniform(-jitter, jitter, X.shape) * hx, 0.0)
    Y = Y + np.where(inner, rng.uniform(-jitter, jitter, Y.shape) * hy, 0.0)
    nodes = np.stack([X.ravel(), Y.ravel()], 1)
    jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    a = (jj * (nx + 1) + ii).ravel()
    b, c, d = a + 1, a + nx + 2, a + nx + 1
    flip = rng.random(a.size) < 0.5
    t1 = np.where(flip[:, None], np.stack([a, b, d], 1), np.stack([a, b, c], 1))
    t2 = np.where(flip[:, None], np.stack([b, c, d], 1), np.stack([a, c, d], 1))
    cells = np.stack([t1, t2], 1).reshape(-1, 3)
    quads = _structured(nodes, nx, ny)
    return from_cells(nodes, cells, quads.bedges, quads.bpatch, quads.patch_names)


def batch_cases(n: int = 256, seed: int = 0, cells=(4096, 65536)):
    """Seeded family of steady airfoil cases for batched solves.

    Per instance: NACA 4-digit section with max camber uniform in [0, 6%]
    (at 40% chord) and thickness uniform in [8%, 18%]; an O-grid whose cell
    count is log-uniform in ``cells`` (ni = 2 nj); freestream Mach uniform in
    [0.3, 0.85] and angle of attack uniform in [-4, 8] degrees.  Returns a
    list of dicts (ni, nj, shape, mach, aoa_deg).
    """
    rng = np.random.default_rng(seed)
    out = []
    lo, hi = np.log(cells[0]), np.log(cells[1])
    for _ in range(n):
        camber = rng.uniform(0.0, 0.06)
        thick = rng.uniform(0.08, 0.18)
        nc = float(np.exp(rng.uniform(lo, hi)))
        nj = max(8, int(round(np.sqrt(nc / 2.0))))
        mach = rng.uniform(0.3, 0.85)
        aoa = rng.uniform(-4.0, 8.0)
        out.append({"ni": 2 * nj, "nj": nj, "shape": (camber, 0.4, thick), "mach": mach, "aoa_deg": aoa})
    return out

