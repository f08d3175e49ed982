"""Polygon meshes and the FVMESH 1.0 text format.

The FVMESH grammar (``# FVMESH 1.0`` header, ``POINTS``/``CELLS``/``BOUNDARY``
sections, CCW cells of any vertex count, boundary edges naming their patch)
is the reference's own interchange format (docs/fvmesh-format.md:12-53,
read by src/MeshReader.cpp:825-958).  Both sides load identical topology from
the same file: coordinates are written with 17 significant digits so every
double round-trips exactly.

Patch numbering follows the reference reader: a patch index is assigned on
the first *matched* boundary edge of each name, in file order
(src/MeshReader.cpp:377-402, :877-892).  ``PolyMesh.patch_names`` is already
in that order when a mesh comes from :func:`read_fvmesh`; the generators in
:mod:`finitevolume_gb300.meshgen` emit boundary edges grouped so that the
order is the listed one.
"""
from __future__ import annotations

import dataclasses
import os
from typing import List

import numpy as np


@dataclasses.dataclass
class PolyMesh:
    """A 2D polygon mesh as node coordinates + CCW cell vertex lists.

    nodes       float64 [n_nodes, 2]
    cell_off    int64   [n_cells + 1]   CSR offsets into ``cell_nodes``
    cell_nodes  int32   [sum of vertex counts]
    bedges      int32   [n_bedges, 2]   boundary edge node pairs
    bpatch      int32   [n_bedges]      patch index of each boundary edge
    patch_names list of str, indexed by patch index
    """

    nodes: np.ndarray
    cell_off: np.ndarray
    cell_nodes: np.ndarray
    bedges: np.ndarray
    bpatch: np.ndarray
    patch_names: List[str]

    @property
    def n_cells(self) -> int:
        return int(self.cell_off.shape[0] - 1)

    @property
    def n_nodes(self) -> int:
        return int(self.nodes.shape[0])

    def cell_sizes(self) -> np.ndarray:
        return np.diff(self.cell_off)

    def patch(self, name: str) -> int:
        return self.patch_names.index(name)

    def validate_ccw(self) -> None:
        """Raise if any cell has non-positive signed (shoelace) area."""
        a = signed_areas(self)
        bad = np.nonzero(~(a > 0.0))[0]
        if bad.size:
            raise ValueError(f"{bad.size} cells have non-positive signed area (first: {bad[0]}, {a[bad[0]]})")


def signed_areas(m: PolyMesh) -> np.ndarray:
    """Vectorised shoelace signed area of every cell."""
    sizes = m.cell_sizes()
    idx = m.cell_nodes.astype(np.int64)
    nxt = np.arange(idx.size) + 1
    ends = m.cell_off[1:] - 1
    nxt[ends] = m.cell_off[:-1]
    p0 = m.nodes[idx]
    p1 = m.nodes[idx[nxt]]
    cross = p0[:, 0] * p1[:, 1] - p1[:, 0] * p0[:, 1]
    cell_of = np.repeat(np.arange(sizes.size), sizes)
    return 0.5 * np.bincount(cell_of, weights=cross, minlength=sizes.size)


def cell_centroids(m: PolyMesh) -> np.ndarray:
    """Shoelace centroids of every cell (signed-area formula), [n_cells, 2]."""
    sizes = m.cell_sizes()
    idx = m.cell_nodes.astype(np.int64)
    nxt = np.arange(idx.size) + 1
    nxt[m.cell_off[1:] - 1] = m.cell_off[:-1]
    p0, p1 = m.nodes[idx], m.nodes[idx[nxt]]
    cross = p0[:, 0] * p1[:, 1] - p1[:, 0] * p0[:, 1]
    cell_of = np.repeat(np.arange(sizes.size), sizes)
    a = 0.5 * np.bincount(cell_of, weights=cross, minlength=sizes.size)
    cx = np.bincount(cell_of, weights=(p0[:, 0] + p1[:, 0]) * cross, minlength=sizes.size) / (6.0 * a)
    cy = np.bincount(cell_of, weights=(p0[:, 1] + p1[:, 1]) * cross, minlength=sizes.size) / (6.0 * a)
    return np.stack([cx, cy], 1)


def from_cells(nodes, cells, bedges, bpatch, patch_names) -> PolyMesh:
    """Build a PolyMesh from a list (or 2D array) of per-cell vertex lists."""
    if isinstance(cells, np.ndarray) and cells.ndim == 2:
        k = cells.shape[1]
        off = np.arange(cells.shape[0] + 1, dtype=np.int64) * k
        flat = cells.reshape(-1).astype(np.int32)
    else:
        sizes = np.fromiter((len(c) for c in cells), dtype=np.int64, count=len(cells))
        off = np.zeros(len(cells) + 1, dtype=np.int64)
        np.cumsum(sizes, out=off[1:])
        flat = np.fromiter((v for c in cells for v in c), dtype=np.int32, count=int(off[-1]))
    return PolyMesh(np.ascontiguousarray(nodes, dtype=np.float64), off, flat,
                    np.ascontiguousarray(bedges, dtype=np.int32).reshape(-1, 2),
                    np.ascontiguousarray(bpatch, dtype=np.int32), list(patch_names))


def write_fvmesh(m: PolyMesh, path: str) -> None:
    """Write ``m`` as FVMESH 1.0 with round-trip-exact coordinates."""
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    with open(path, "w") as f:
        f.write("# FVMESH 1.0\n")
        f.write(f"POINTS {m.n_nodes}\n")
        np.savetxt(f, m.nodes, fmt="%.17g")
        f.write(f"CELLS {m.n_cells}\n")
        sizes = m.cell_sizes()
        # Group cells by vertex count so each block is a rectangular savetxt.
        lines = np.empty(m.n_cells, dtype=object)
        for k in np.unique(sizes):
            sel = np.nonzero(sizes == k)[0]
            rows = m.cell_nodes[(m.cell_off[sel][:, None] + np.arange(k)[None, :])]
            block = np.concatenate([np.full((sel.size, 1), k, dtype=np.int64), rows], axis=1)
            txt = [" ".join(map(str, r)) for r in block.tolist()]
            lines[sel] = txt
        f.write("\n".join(lines.tolist()))
        f.write("\n")
        f.write(f"BOUNDARY {m.bedges.shape[0]}\n")
        names = np.asarray(m.patch_names, dtype=object)[m.bpatch]
        f.write("\n".join(f"{a} {b} {n}" for (a, b), n in zip(m.bedges.tolist(), names.tolist())))
        f.write("\n")


def read_fvmesh(path: str) -> PolyMesh:
    """Parse FVMESH 1.0 (docs/fvmesh-format.md) into a PolyMesh.

    Patch indices follow the reference reader's lazy numbering: patches are
    numbered in order of their first boundary edge that matches a cell edge
    (src/MeshReader.cpp:377-402); edges that match no cell edge are dropped,
    as the reference silently ignores them (src/MeshReader.cpp:380).
    """
    with open(path) as f:
        header = f.readline().split()
        if len(header) < 3 or header[0] != "#" or header[1] != "FVMESH" or header[2] != "1.0":
            raise ValueError(f"{path}: unsupported FVMESH header {header}")
        tokens = f.read().split()
    pos = 0
    nodes = cells_flat = None
    sizes = None
    bedges, bnames = [], []
    while pos < len(tokens):
        tag = tokens[pos]
        count = int(tokens[pos + 1])
        pos += 2
        if tag == "POINTS":
            nodes = np.array(tokens[pos:pos + 2 * count], dtype=np.float64).reshape(count, 2)
            pos += 2 * count
        elif tag == "CELLS":
            sz = np.empty(count, dtype=np.int64)
            flat = []
            for i in range(count):
                k = int(tokens[pos])
                sz[i] = k
                flat.extend(tokens[pos + 1:pos + 1 + k])
                pos += 1 + k
            sizes = sz
            cells_flat = np.array(flat, dtype=np.int32)
        elif tag == "BOUNDARY":
            for i in range(count):
                bedges.append((int(tokens[pos]), int(tokens[pos + 1])))
                bnames.append(tokens[pos + 2])
                pos += 3
        else:
            raise ValueError(f"{path}: unrecognised section {tag}")
    off = np.zeros(sizes.size + 1, dtype=np.int64)
    np.cumsum(sizes, out=off[1:])
    # Edge set of all cells, to reproduce the reader's "match or drop" rule.
    idx = cells_flat.astype(np.int64)
    nxt = np.arange(idx.size) + 1
    nxt[off[1:] - 1] = off[:-1]
    a, b = idx, idx[nxt]
    keys = set((np.minimum(a, b) * (1 << 32) + np.maximum(a, b)).tolist())
    names: List[str] = []
    kept_e, kept_p = [], []
    for (u, v), n in zip(bedges, bnames):
        if (min(u, v) << 32) + max(u, v) not in keys:
            continue
        if n not in names:
            names.append(n)
        kept_e.append((u, v))
        kept_p.append(names.index(n))
    return PolyMesh(nodes, off, cells_flat, np.array(kept_e, dtype=np.int32).reshape(-1, 2),
                    np.array(kept_p, dtype=np.int32), names)
