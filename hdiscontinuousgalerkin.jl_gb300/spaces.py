"""Finite elements and function spaces of the HDG path (src/basis.jl, src/FiniteElement.jl,
src/ScalarFunctionSpaces.jl, src/VectorFunctionSpaces.jl, src/TraceFunctionSpaces.jl).

The three spaces of one HDG discretisation share one libhdg space handle (the mesh, the degree
and the quadrature rules are common); the reference tables live on the device.  The per-cell
accessors (reinit!, shape_value, getdetJdV, ...) are host conveniences for user code that
inspects a cell; the assembly itself runs on the device (see system.py)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


class RefTetrahedron:
    """Reference triangle (0,0),(1,0),(0,1) (src/shapes.jl)."""


class Dubiner:
    """Dubiner{2,RefTetrahedron,order}: orthonormal modal basis (src/basis.jl:50-123)."""

    def __init__(self, dim: int = 2, shape=RefTetrahedron, order: int = 1):
        if dim != 2:
            raise ValueError("Dubiner is 2D")
        self.dim, self.shape, self.order = dim, shape, int(order)

    def getnbasefunctions(self):
        return (self.order + 1) * (self.order + 2) // 2


class Legendre:
    """Legendre{1,RefTetrahedron,order}: orthonormal on (0,1) (src/basis.jl:341-364)."""

    def __init__(self, dim: int = 1, shape=RefTetrahedron, order: int = 1):
        if dim != 1:
            raise ValueError("Legendre is 1D")
        self.dim, self.shape, self.order = dim, shape, int(order)

    def getnbasefunctions(self):
        return self.order + 1


class GenericFiniteElement:
    """GenericFiniteElement(func_basis) with P1 Lagrange geometry (src/FiniteElement.jl:8-27)."""

    def __init__(self, basis):
        self.basis = basis
        self.order = basis.order

    def getnbasefunctions(self):
        return self.basis.getnbasefunctions()


class ContinuousLagrange:
    """ContinuousLagrange{dim,RefTetrahedron,order}: nodal P_order element with P1 geometry
    (src/LagrangeFE.jl:5-61).  Nodes are ordered as get_nodal_points of src/shapes.jl:46-77:
    the three vertices, then the order-1 interior points of each reference edge (1,0)->(0,1),
    (0,1)->(0,0), (0,0)->(1,0), then the interior points.  topology[k] counts the dofs on
    entities of dimension k."""

    EDGES = (((1.0, 0.0), (0.0, 1.0)), ((0.0, 1.0), (0.0, 0.0)), ((0.0, 0.0), (1.0, 0.0)))

    def __init__(self, dim: int = 2, shape=RefTetrahedron, order: int = 1):
        if dim != 2 or order < 1:
            raise ValueError("ContinuousLagrange is implemented for triangles (dim 2), order >= 1")
        self.dim, self.shape, self.order = dim, shape, int(order)
        k = self.order
        self.topology = {0: 3, 1: 3 * (k - 1), 2: (k - 1) * (k - 2) // 2}

    def getnbasefunctions(self):
        return (self.order + 1) * (self.order + 2) // 2

    def nodal_points(self):
        k = self.order
        pts = [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0)]
        for a, b in self.EDGES:
            for i in range(1, k):
                pts.append((a[0] + i * (b[0] - a[0]) / k, a[1] + i * (b[1] - a[1]) / k))
        for i in range(1, k):            # interior grid, src/shapes.jl:_interior_points (m = 2):
            for j in range(1, k - i):    # v1 + i (v3 - v1)/k + j (v2 - v1)/k
                pts.append((j / k, i / k))
        return np.array(pts)

    def spatial_nodal_coordinate(self, i: int, coords):
        """x of local node i (1-based) on a cell with vertex coordinates coords (3 x 2), P1 map."""
        xi, eta = self.nodal_points()[i - 1]
        c = np.asarray(coords, dtype=float)
        return (1.0 - xi - eta) * c[0] + xi * c[1] + eta * c[2]


_space_cache = {}


class _SpaceHandle:
    def __init__(self, mesh, p: int, qd: int):
        self.mesh = mesh
        h = C.c_void_p()
        L.check(L.load().hdg_space_create(mesh.handle, int(p), int(qd), C.byref(h)), mesh.ctx)
        self.h = h
        lib = L.load()
        v = [C.c_int() for _ in range(5)]
        L.check(lib.hdg_space_info(self.h, *[C.byref(x) for x in v]))
        self.nw, self.nv, self.nt, self.nq, self.nfq = (x.value for x in v)
        self.p, self.qd = p, qd
        self.pts = np.zeros((self.nq, 2))
        self.w = np.zeros(self.nq)
        self.N = np.zeros((self.nw, self.nq))
        self.dN = np.zeros((self.nw, self.nq, 2))
        self.fpts = np.zeros(self.nfq)
        self.fw = np.zeros(self.nfq)
        self.E = np.zeros((self.nw, self.nfq, 3))
        self.T = np.zeros((self.nt, self.nfq))
        L.check(lib.hdg_space_tables(self.h, *[L.dptr(a) for a in (self.pts, self.w, self.N, self.dN, self.fpts, self.fw,
                                                                   self.E, self.T)]))

    def __del__(self):
        try:
            if self.h:
                L.load().hdg_space_destroy(self.h)
        except Exception:
            pass

    def geometry(self, cell: int):
        detJ = C.c_double()
        Jinv, detJf, nrm = np.zeros(4), np.zeros(3), np.zeros(6)
        L.check(L.load().hdg_space_cell_geometry(self.h, int(cell), C.byref(detJ), L.dptr(Jinv), L.dptr(detJf),
                                                 L.dptr(nrm)), self.mesh.ctx)
        return detJ.value, Jinv.reshape(2, 2), detJf, nrm.reshape(3, 2)


def _handle(mesh, p, qd):
    key = (id(mesh), p, qd)
    h = _space_cache.get(key)
    if h is None or h.mesh is not mesh:
        h = _SpaceHandle(mesh, p, qd)
        _space_cache[key] = h
    return h


class _CellState:
    """Per-cell geometry of the last reinit! (detJ, Jinv, detJf, normals)."""

    def __init__(self):
        self.detJ = np.nan
        self.Jinv = np.full((2, 2), np.nan)
        self.detJf = np.full(3, np.nan)
        self.normals = np.full((3, 2), np.nan)


class ScalarFunctionSpace:
    """ScalarFunctionSpace(mesh, fe; quad_degree = order+1) (src/ScalarFunctionSpaces.jl:24-29)."""

    def __init__(self, mesh, fe, update_face_data: bool = True, quad_degree: int | None = None):
        self.mesh, self.fe = mesh, fe
        self.order = fe.order
        self.quad_degree = quad_degree if quad_degree is not None else fe.order + 1
        # nodal (continuous Lagrange) spaces only carry dofs for a DofHandler; the HDG tables
        # live in the device space handle of the modal (Dubiner) spaces
        self.sp = None if isinstance(fe, ContinuousLagrange) else _handle(mesh, self.order, self.quad_degree)
        self.state = _CellState()

    def getnbasefunctions(self):
        return self.fe.getnbasefunctions() if self.sp is None else self.sp.nw

    def getnlocaldofs(self):
        return self.getnbasefunctions()

    def getnquadpoints(self):
        return self.sp.nq

    def getnfacequadpoints(self):
        return self.sp.nfq


class VectorFunctionSpace(ScalarFunctionSpace):
    """VectorFunctionSpace(mesh, fe): [P_p]^2, component-major dofs (src/VectorFunctionSpaces.jl:10-18)."""

    def getnbasefunctions(self):
        return 2 * self.sp.nw

    def getnlocaldofs(self):
        return 2 * self.sp.nw


class ScalarTraceFunctionSpace:
    """ScalarTraceFunctionSpace(Wh, fe_trace) (src/TraceFunctionSpaces.jl:11-28)."""

    def __init__(self, parent: ScalarFunctionSpace, fe):
        if fe.order != parent.order:
            raise NotImplementedError("the GPU path uses trace degree = volume degree, as the reference example does")
        self.fs, self.fe, self.mesh = parent, fe, parent.mesh
        self.sp = parent.sp
        self.order = fe.order

    def getnbasefunctions(self):
        return self.sp.nt

    def getnlocaldofs(self):
        return 3 * self.sp.nt

    def getnquadpoints(self):
        return self.sp.nfq


# ---- per-cell accessors (host) --------------------------------------------------------------
def getnbasefunctions(x):
    return x.getnbasefunctions()


def getnlocaldofs(x):
    return x.getnlocaldofs()


def getnquadpoints(fs):
    return fs.getnquadpoints()


def getnfacequadpoints(fs):
    return fs.sp.nfq


def reinit_(fs, cell):
    """reinit!(fs, cell): cell geometry of a 1-based cell index (or a CellIterator state)."""
    idx = cell if isinstance(cell, int) else cell.current_cellid
    st = fs.state if hasattr(fs, "state") else fs.fs.state
    st.detJ, st.Jinv, st.detJf, st.normals = fs.sp.geometry(idx)
    return fs


def getdetJdV(fs, q_point: int) -> float:
    return fs.state.detJ * fs.sp.w[q_point - 1]


def getfacedetJdS(fs, face: int, q_point: int) -> float:
    st = fs.state if hasattr(fs, "state") else fs.fs.state
    return st.detJf[face - 1] * fs.sp.fw[q_point - 1]


def get_normal(fs, face: int):
    return fs.state.normals[face - 1].copy()


def shape_value(fs, *args):
    """shape_value(fs, q, i) / shape_value(fs, face, q, i[, orientation]) with 1-based indices."""
    sp = fs.sp
    if isinstance(fs, ScalarTraceFunctionSpace):
        q, i = args
        return sp.T[i - 1, q - 1]
    vector = isinstance(fs, VectorFunctionSpace)
    if len(args) == 2:
        q, i = args
        if vector:
            v = np.zeros(2)
            v[(i - 1) // sp.nw] = sp.N[(i - 1) % sp.nw, q - 1]
            return v
        return sp.N[i - 1, q - 1]
    face, q, i = args[:3]
    orient = args[3] if len(args) > 3 else True
    qq = q - 1 if orient else sp.nfq - q
    if vector:
        v = np.zeros(2)
        v[(i - 1) // sp.nw] = sp.E[(i - 1) % sp.nw, qq, face - 1]
        return v
    return sp.E[i - 1, qq, face - 1]


def shape_gradient(fs, q: int, i: int):
    sp, Jinv = fs.sp, fs.state.Jinv
    if isinstance(fs, VectorFunctionSpace):
        G = np.zeros((2, 2))
        G[(i - 1) // sp.nw, :] = sp.dN[(i - 1) % sp.nw, q - 1]
        return G @ Jinv
    return sp.dN[i - 1, q - 1] @ Jinv


def shape_divergence(fs, q: int, i: int) -> float:
    g = shape_gradient(fs, q, i)
    return float(np.trace(g)) if g.ndim == 2 else float(g.sum())
