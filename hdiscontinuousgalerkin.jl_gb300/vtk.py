"""Headless output of a solution for visualisation: a legacy-format VTK unstructured grid.

The reference's example ends by plotting u with Makie (`examples/poisson2D_HDG.jl:214-216`, the
per-node averages of `nodal_avg`, `src/DiscreteFunctions.jl:81-95`).  No graphics stack is
available here, so the same data goes to a file that any VTK reader opens:

    write_vtk("u.vtk", mesh, point_data={"u": nodal_avg(u_h)}, cell_data={"kappa": kc})
"""
from __future__ import annotations

import numpy as np


def write_vtk(path: str, mesh, point_data: dict | None = None, cell_data: dict | None = None,
              title: str = "hdg") -> None:
    """Write the triangles of `mesh` (nodes in the plane z = 0) with scalar or 2-vector fields
    per node (`point_data`, arrays of length nnodes) and per cell (`cell_data`, length ncells)."""
    xy, cells = mesh._topology()[0], mesh._topology()[1]
    nn, nc = xy.shape[0], cells.shape[0]
    out = [f"# vtk DataFile Version 3.0\n{title}\nASCII\nDATASET UNSTRUCTURED_GRID\n",
           f"POINTS {nn} double\n"]
    out += [f"{x:.17g} {y:.17g} 0\n" for x, y in xy]
    out.append(f"CELLS {nc} {4 * nc}\n")
    out += [f"3 {a - 1} {b - 1} {c - 1}\n" for a, b, c in cells]  # 1-based ids -> 0-based
    out.append(f"CELL_TYPES {nc}\n")
    out.append("5\n" * nc)

    def block(kind, n, fields):
        if not fields:
            return
        out.append(f"{kind} {n}\n")
        for name, val in fields.items():
            v = np.asarray(val, dtype=np.float64)
            if v.shape[0] != n:
                raise ValueError(f"{name}: expected {n} values, got {v.shape[0]}")
            if v.ndim == 1:
                out.append(f"SCALARS {name} double 1\nLOOKUP_TABLE default\n")
                out.extend(f"{x:.17g}\n" for x in v)
            elif v.ndim == 2 and v.shape[1] == 2:
                out.append(f"VECTORS {name} double\n")
                out.extend(f"{a:.17g} {b:.17g} 0\n" for a, b in v)
            else:
                raise ValueError(f"{name}: scalars or 2-vectors only")

    block("POINT_DATA", nn, point_data)
    block("CELL_DATA", nc, cell_data)
    with open(path, "w") as fh:
        fh.write("".join(out))
