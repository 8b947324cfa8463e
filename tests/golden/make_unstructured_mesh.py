"""Writes a large unstructured triangle mesh of the unit square in Triangle's file format
(.node/.ele/.edge), for the at-scale test of parse_mesh_triangle (src/triangle_mesh.jl:115-126).

The points are an m x m grid with every interior point moved by U(-0.3h, 0.3h) per coordinate
(seeded) and the points on the four sides moved along their side only; the cells are their
Delaunay triangulation (scipy.spatial.Delaunay), turned counter-clockwise.  About 2 m^2 cells:
m = 225 gives about 100k.  Every edge is listed in .edge with boundary marker 1 on the square's
sides and 0 inside, which is how the reference's reader finds the "boundary" face set.  Numbers are
written in plain decimal notation (no sign, no exponent), the only form the reference's reader
(read_line, src/triangle_mesh.jl:2-5) accepts.

    python tests/golden/make_unstructured_mesh.py <root> [m] [seed]
"""
from __future__ import annotations

import sys

import numpy as np


def unstructured_square(m: int = 225, seed: int = 2024):
    """(xy [nn x 2], cells [nc x 3] 0-based counter-clockwise, edges [ne x 2] 0-based, boundary [ne])."""
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    h = 1.0 / (m - 1)
    g = np.linspace(0.0, 1.0, m)
    X, Y = np.meshgrid(g, g, indexing="xy")
    xy = np.column_stack([X.ravel(), Y.ravel()])
    d = rng.uniform(-0.3 * h, 0.3 * h, xy.shape)
    on_x = (xy[:, 0] == 0.0) | (xy[:, 0] == 1.0)
    on_y = (xy[:, 1] == 0.0) | (xy[:, 1] == 1.0)
    d[on_x, 0] = 0.0          # points on x = 0, 1 move along y only
    d[on_y, 1] = 0.0          # points on y = 0, 1 move along x only
    d[on_x & on_y] = 0.0      # corners stay
    xy = xy + d
    tri = Delaunay(xy).simplices.astype(np.int64)
    a, b, c = xy[tri[:, 0]], xy[tri[:, 1]], xy[tri[:, 2]]
    area2 = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    tri = tri[area2 != 0.0]
    area2 = area2[area2 != 0.0]
    flip = area2 < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    # cells in rows of the grid, left to right (the spatially coherent order a mesh generator
    # writes), so that first-visit face numbering gives the trace matrix a narrow band
    cen = xy[tri].mean(axis=1)
    tri = tri[np.lexsort((cen[:, 0], np.floor(cen[:, 1] / h)))]
    e = np.sort(np.concatenate([tri[:, [1, 2]], tri[:, [2, 0]], tri[:, [0, 1]]]), axis=1)
    edges, count = np.unique(e, axis=0, return_counts=True)
    boundary = (count == 1).astype(np.int64)
    return xy, tri, edges, boundary


def write_triangle_mesh(root: str, m: int = 225, seed: int = 2024):
    """Writes root.node, root.ele, root.edge; returns the number of cells."""
    xy, tri, edges, boundary = unstructured_square(m, seed)
    nb = np.zeros(len(xy), np.int64)
    nb[edges[boundary == 1].ravel()] = 1
    with open(root + ".node", "w") as fh:
        fh.write(f"{len(xy)}  2  0  1\n")
        fh.writelines(f"{i + 1} {x:.17f} {y:.17f} {b}\n" for i, ((x, y), b) in enumerate(zip(xy, nb)))
    with open(root + ".ele", "w") as fh:
        fh.write(f"{len(tri)}  3  0\n")
        fh.writelines(f"{i + 1} {t[0] + 1} {t[1] + 1} {t[2] + 1}\n" for i, t in enumerate(tri))
    with open(root + ".edge", "w") as fh:
        fh.write(f"{len(edges)}  1\n")
        fh.writelines(f"{i + 1} {v[0] + 1} {v[1] + 1} {b}\n" for i, (v, b) in enumerate(zip(edges, boundary)))
    return len(tri)


if __name__ == "__main__":
    root = sys.argv[1]
    m = int(sys.argv[2]) if len(sys.argv) > 2 else 225
    seed = int(sys.argv[3]) if len(sys.argv) > 3 else 2024
    print(write_triangle_mesh(root, m, seed), "cells")
