"""DofHandler, sparsity patterns and the sparsity-pattern assembler (src/dofhandler.jl,
src/assembler.jl:62-137), over libhdg's host implementation (csrc/dofhandler.cpp).

    dh = DofHandler([u_h], mesh)                 # first-visit vertex / face / cell numbering
    dh.cell_dofs, dh.cell_dofs_offset            # 1-based, as the reference stores them
    K = create_sparsity_pattern(dh)              # scipy CSC with stored zeros
    A = start_assemble(K, f); assemble_(A, celldofs, Ke, fe)
    dbc = Dirichlet(u_h, dh, "boundary", g)      # nodal values of g on the face set

These serve nodal (continuous Lagrange) fields; the HDG path numbers its trace dofs face-major
without a DofHandler (examples/poisson2D_HDG.jl:176-181)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .spaces import ContinuousLagrange


def _check(rc):
    if rc != L.HDG_OK:
        msg = L.load().hdg_dofhandler_last_error()
        raise L.HDGError(rc, msg.decode() if msg else "")


def _field_topology(u):
    """(dofs per vertex, per face, per cell, components) of a TrialFunction's element:
    gettopology(fe)[k] divided by the reference triangle's entity counts (3, 3, 1)."""
    fe = u.fs.fe
    if not isinstance(fe, ContinuousLagrange):
        raise NotImplementedError("DofHandler numbers nodal fields (ContinuousLagrange)")
    t = fe.topology
    for k, ne in ((0, 3), (1, 3)):
        if t[k] % ne:
            raise ValueError("element topology is not divisible by the cell's entity count")
    return t[0] // 3, t[1] // 3, t[2], int(getattr(u, "ncomponents", 1))


class DofHandler:
    """DofHandler(fields, mesh) (src/dofhandler.jl:13-16)."""

    def __init__(self, variables, mesh):
        self.variables = list(variables)
        self.mesh = mesh
        topo = [_field_topology(u) for u in self.variables]
        arr = [(C.c_int * len(topo))(*[t[i] for t in topo]) for i in range(4)]
        h = C.c_void_p()
        _check(L.load().hdg_dofhandler_create(mesh.handle, len(topo), *arr, C.byref(h)))
        self.h = h
        nd, nc = C.c_int(), C.c_int64()
        _check(L.load().hdg_dofhandler_sizes(self.h, C.byref(nd), C.byref(nc)))
        self._ndofs = nd.value
        self.cell_dofs = np.zeros(nc.value, np.int32)
        self.cell_dofs_offset = np.zeros(mesh.ncells + 1, np.int32)
        _check(L.load().hdg_dofhandler_cell_dofs(self.h, L.i32ptr(self.cell_dofs), L.i32ptr(self.cell_dofs_offset)))

    def __del__(self):
        try:
            if self.h:
                L.load().hdg_dofhandler_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def ndofs(self) -> int:
        return self._ndofs

    def ndofs_per_cell(self, cell: int = 1) -> int:
        return int(self.cell_dofs_offset[cell] - self.cell_dofs_offset[cell - 1])

    def nvariables(self) -> int:
        return len(self.variables)

    def find_field(self, field) -> int:
        for i, v in enumerate(self.variables):
            if v is field:
                return i
        raise KeyError(f"did not find field {field}")


def ndofs(dh: DofHandler) -> int:
    return dh.ndofs()


def ndofs_per_cell(dh: DofHandler, cell: int = 1) -> int:
    return dh.ndofs_per_cell(cell)


def nvariables(dh: DofHandler) -> int:
    return dh.nvariables()


def celldofs_(global_dofs, dh: DofHandler, i: int):
    """celldofs!(global_dofs, dh, i): dofs of cell i (1-based) into global_dofs."""
    a, b = dh.cell_dofs_offset[i - 1] - 1, dh.cell_dofs_offset[i] - 1
    if len(global_dofs) != b - a:
        raise ValueError("global_dofs has the wrong length")
    global_dofs[:] = dh.cell_dofs[a:b]
    return global_dofs


def dof_range(dh: DofHandler, field) -> range:
    """Local dof range of a field within a cell (1-based, inclusive like Julia's a:b)."""
    first, last = C.c_int(), C.c_int()
    _check(L.load().hdg_dofhandler_field_range(dh.h, dh.find_field(field), C.byref(first), C.byref(last)))
    return range(first.value, last.value + 1)


def _sparsity(dh: DofHandler, symmetric: bool):
    import scipy.sparse as sp
    nnz = C.c_int64()
    _check(L.load().hdg_dofhandler_sparsity(dh.h, int(symmetric), 0, None, None, C.byref(nnz)))
    colptr = np.zeros(dh.ndofs() + 1, np.int64)
    rowval = np.zeros(nnz.value, np.int64)
    _check(L.load().hdg_dofhandler_sparsity(dh.h, int(symmetric), 0, L.i64ptr(colptr), L.i64ptr(rowval),
                                            C.byref(nnz)))
    return sp.csc_matrix((np.zeros(nnz.value), rowval, colptr), shape=(dh.ndofs(), dh.ndofs()))


def create_sparsity_pattern(dh: DofHandler):
    """create_sparsity_pattern(dh) (src/dofhandler.jl:171): CSC with every stored entry 0."""
    return _sparsity(dh, False)


def create_symmetric_sparsity_pattern(dh: DofHandler):
    """create_symmetric_sparsity_pattern(dh) (src/dofhandler.jl:184): upper triangle only."""
    return _sparsity(dh, True)


class AssemblerSparsityPattern:
    """start_assemble(K, f) on a stored pattern (src/assembler.jl:62-86): assemble_ adds element
    matrices into K.data in place and element vectors into f."""

    def __init__(self, K, f=None, symmetric: bool = False):
        K.sort_indices()
        self.K, self.f, self.symmetric = K, f, symmetric
        self.K.data[:] = 0.0
        if f is not None:
            f[:] = 0.0


def start_assemble(K, f=None, symmetric: bool = False):
    return AssemblerSparsityPattern(K, f, symmetric)


def assemble_(A: AssemblerSparsityPattern, dofs, Ke, fe=None):
    """assemble!(A, dofs, Ke[, fe]) (src/assembler.jl:97-137).  dofs are 1-based; dofs may be a
    batch (nel x n) with Ke (nel x n x n) and fe (nel x n)."""
    d = np.ascontiguousarray(dofs, dtype=np.int64)
    Kt = np.asarray(Ke, dtype=np.float64)
    one = d.ndim == 1
    if one:
        d = d[None, :]
        Kt = Kt[None, :, :]
    nel, n = d.shape
    Kcm = np.ascontiguousarray(np.transpose(Kt, (0, 2, 1)))  # column-major element matrices
    fa = None
    if fe is not None and len(np.ravel(fe)):
        fa = np.ascontiguousarray(np.reshape(fe, (nel, n)), dtype=np.float64)
        if A.f is None:
            raise ValueError("the assembler was started without f")
    K = A.K
    rc = L.load().hdg_csc_assemble(K.shape[0], L.i64ptr(np.ascontiguousarray(K.indptr, dtype=np.int64)),
                                   L.i64ptr(np.ascontiguousarray(K.indices, dtype=np.int64)), 0,
                                   K.data.ctypes.data_as(L.dp), L.dptr(A.f) if fa is not None else None,
                                   int(A.symmetric), nel, n, L.i64ptr(d), L.dptr(Kcm), L.dptr(fa))
    _check(rc)


class DirichletDH:
    """Dirichlet(u, dh, faceset, g) for a nodal field (src/boundary.jl:44-95): the field's vertex
    and face dofs on the face set, sorted, with g evaluated at their nodal points.  g is a
    callable of a 2-vector (returning a scalar or one value per component), a Field, or a vector
    of per-component values."""

    def __init__(self, u, dh: DofHandler, faceset: str, g):
        fi = dh.find_field(u)
        n = C.c_int()
        _check(L.load().hdg_dofhandler_dirichlet(dh.h, faceset.encode(), fi, None, None, None, C.byref(n)))
        dofs, cells, loc = (np.zeros(n.value, np.int32) for _ in range(3))
        _check(L.load().hdg_dofhandler_dirichlet(dh.h, faceset.encode(), fi, L.i32ptr(dofs), L.i32ptr(cells),
                                                 L.i32ptr(loc), C.byref(n)))
        ncomp = int(getattr(u, "ncomponents", 1))
        if ncomp != 1:
            raise NotImplementedError("Dirichlet on a DofHandler prescribes scalar nodal fields")
        xy = dh.mesh._topology()[0]
        cn = dh.mesh._topology()[1]
        fe = u.fs.fe
        vals = []
        for c, i in zip(cells, loc):
            if callable(g):
                x = fe.spatial_nodal_coordinate(int(i), xy[cn[c - 1] - 1])
                v = np.atleast_1d(g(x) if not hasattr(g, "kind") else g(x[0], x[1]))
            else:
                v = np.atleast_1d(np.asarray(g, dtype=float))
            vals.append(float(v[0]))
        self.prescribed_dofs = dofs.astype(np.int64)
        self.values = np.asarray(vals)
