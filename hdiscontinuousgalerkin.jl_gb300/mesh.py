"""Meshes: rectangle_mesh and parse_mesh_triangle (src/generate_mesh.jl, src/triangle_mesh.jl,
src/mesh.jl), held by libhdg with a device copy of the topology."""
from __future__ import annotations

import ctypes as C
import re
from collections import namedtuple

import numpy as np

from . import _lib as L
from .context import default_context

Cell = namedtuple("Cell", ["nodes", "faces"])  # 1-based ids, src/mesh.jl:17-20
Node = namedtuple("Node", ["x"])


class TriangleCell:
    """Cell{2,3,3}: marker type for rectangle_mesh(TriangleCell, ...), src/mesh.jl:24."""
    reference_edge_nodes = ((2, 3), (3, 1), (1, 2))


class PolygonalMesh:
    """PolygonalMesh{2,3,3,2,Float64} (src/mesh.jl:43-49) backed by an hdg_mesh handle."""

    def __init__(self, handle, ctx):
        self._h = handle
        self.ctx = ctx
        lib = L.load()
        nn, nc, nf = C.c_int(), C.c_int(), C.c_int()
        L.check(lib.hdg_mesh_sizes(self._h, C.byref(nn), C.byref(nc), C.byref(nf)))
        self.nnodes, self.ncells, self.nfaces = nn.value, nc.value, nf.value
        self._topo = None

    @property
    def handle(self):
        return self._h

    def __del__(self):
        try:
            if self._h:
                L.load().hdg_mesh_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def _topology(self):
        if self._topo is None:
            xy = np.zeros((self.nnodes, 2))
            cn = np.zeros((self.ncells, 3), np.int32)
            cf = np.zeros((self.ncells, 3), np.int32)
            fc = np.zeros((self.nfaces, 4), np.int32)
            L.check(L.load().hdg_mesh_get_topology(self._h, L.dptr(xy), L.i32ptr(cn), L.i32ptr(cf), L.i32ptr(fc)))
            self._topo = (xy, cn, cf, fc)
        return self._topo

    # ---- the reference's accessors ------------------------------------------------------
    @property
    def cells(self):
        _, cn, cf, _ = self._topology()
        return [Cell(tuple(int(v) for v in a), tuple(int(v) for v in b)) for a, b in zip(cn, cf)]

    @property
    def nodes(self):
        return [Node(tuple(x)) for x in self._topology()[0]]

    @property
    def faces(self):
        """rows [v1 v2 cell1 cell2] (1-based, cell2 = 0 on the boundary)."""
        return self._topology()[3].copy()

    def set_coordinates(self, xy):
        xy = L.f64(xy).reshape(self.nnodes, 2)
        L.check(L.load().hdg_mesh_set_coordinates(self._h, L.dptr(xy)), self.ctx)
        self._topo = None

    def jitter(self, a: float, seed: int):
        """Move interior nodes by U(-a, a) * h per coordinate (rectangle meshes only)."""
        L.check(L.load().hdg_mesh_jitter(self._h, float(a), int(seed)), self.ctx)
        self._topo = None


def getncells(mesh):
    return mesh.ncells


def getnnodes(mesh):
    return mesh.nnodes


def getnfaces(mesh_or_cell):
    if isinstance(mesh_or_cell, Cell):
        return len(mesh_or_cell.faces)
    return mesh_or_cell.nfaces


def n_faces_per_cell(mesh):
    return 3


def getcells_matrix(mesh):
    return mesh._topology()[1].copy()


def get_vertices_matrix(mesh):
    return mesh._topology()[0].copy()


def getfaceset(mesh, name: str):
    lib = L.load()
    n = C.c_int()
    L.check(lib.hdg_mesh_faceset(mesh.handle, name.encode(), None, C.byref(n)), mesh.ctx)
    out = np.zeros(max(n.value, 1), np.int32)
    L.check(lib.hdg_mesh_faceset(mesh.handle, name.encode(), L.i32ptr(out), C.byref(n)), mesh.ctx)
    return set(int(v) for v in out[: n.value])


def face_orientation(mesh, cell_idx: int, face_idx: int) -> bool:
    """face_orientation(mesh, cell, face) (src/mesh.jl:51-54), 1-based indices."""
    k = TriangleCell.reference_edge_nodes[face_idx - 1]
    nodes = mesh._topology()[1][cell_idx - 1]
    return bool(nodes[k[1] - 1] > nodes[k[0] - 1])


def get_coordinates(cell, mesh):
    xy = mesh._topology()[0]
    return [tuple(xy[n - 1]) for n in cell.nodes]


def cell_diameter(mesh, idx: int) -> float:
    """Longest face of cell idx (src/mesh.jl:126-134)."""
    xy, _, cf, fc = mesh._topology()
    h = 0.0
    for f in cf[idx - 1]:
        v1, v2 = fc[f - 1, 0], fc[f - 1, 1]
        h = max(h, float(np.linalg.norm(xy[v2 - 1] - xy[v1 - 1])))
    return h


def rectangle_mesh(cell_type, nel, LL=(0.0, 0.0), UR=(1.0, 1.0), ctx="default") -> PolygonalMesh:
    """rectangle_mesh(TriangleCell, (nx, ny), LL, UR) (src/generate_mesh.jl:101-143).
    ctx=None builds a host-only mesh (topology queries only)."""
    if cell_type is not TriangleCell:
        raise NotImplementedError("only TriangleCell meshes are on the HDG path")
    ctx = default_context() if ctx == "default" else ctx
    h = C.c_void_p()
    ll, ur = L.f64(LL), L.f64(UR)
    L.check(L.load().hdg_mesh_rectangle(ctx.handle if ctx else None, int(nel[0]), int(nel[1]), L.dptr(ll), L.dptr(ur),
                                        C.byref(h)), ctx.handle if ctx else None)
    return PolygonalMesh(h, ctx.handle if ctx else None)


_NUM = re.compile(r"\b((\d*\.)?\d+)\b")


def _records(path):
    first = True
    with open(path) as fh:
        for ln in fh:
            if re.match(r"^\s*(?:#|$)", ln):
                continue
            if first:
                first = False
                continue
            yield [m.group(0) for m in _NUM.finditer(ln)]


def parse_mesh_triangle(root_file: str, ctx="default") -> PolygonalMesh:
    """parse_mesh_triangle(root_file) (src/triangle_mesh.jl:115-126): .node, .edge, .ele files."""
    nodes = [(float(r[1]), float(r[2])) for r in _records(root_file + ".node")]
    edges = [(int(r[1]), int(r[2]), int(r[3])) for r in _records(root_file + ".edge")]
    cells = [(int(r[1]), int(r[2]), int(r[3])) for r in _records(root_file + ".ele")]
    ctx = default_context() if ctx == "default" else ctx
    xy, cl, ed = L.f64(nodes), L.i32(cells), L.i32(edges)
    h = C.c_void_p()
    L.check(L.load().hdg_mesh_from_cells(ctx.handle if ctx else None, len(xy), L.dptr(xy), len(cl), L.i32ptr(cl),
                                         len(ed), L.i32ptr(ed), C.byref(h)), ctx.handle if ctx else None)
    return PolygonalMesh(h, ctx.handle if ctx else None)
