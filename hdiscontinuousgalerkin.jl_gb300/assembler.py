"""start_assemble / assemble! / end_assemble (src/assembler.jl:1-60) for user-written element
loops: triplets collected by libhdg's host assembler, finished into CSC with duplicates summed."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


class Assembler:
    def __init__(self, sizehint: int = 0):
        h = C.c_void_p()
        L.check(L.load().hdg_assembler_create(int(sizehint), C.byref(h)))
        self._h = h

    def __del__(self):
        try:
            if self._h:
                L.load().hdg_assembler_destroy(self._h)
        except Exception:
            pass


class SparseMatrixCSC:
    """Host CSC matrix (1-based colptr/rowval like Julia's SparseMatrixCSC when base=1)."""

    def __init__(self, m, n, colptr, rowval, nzval):
        self.m, self.n = m, n
        self.colptr, self.rowval, self.nzval = colptr, rowval, nzval

    @property
    def shape(self):
        return (self.m, self.n)

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csc_matrix((self.nzval, self.rowval - 1, self.colptr - 1), shape=self.shape)


def start_assemble(N=0, f=None, symmetric: bool = False):
    """start_assemble(N) -> triplet Assembler (src/assembler.jl:23-29), or start_assemble(K, f)
    on a stored sparsity pattern K (scipy CSC from create_sparsity_pattern) -> an in-place
    assembler (src/assembler.jl:72-86)."""
    if hasattr(N, "indptr"):
        from .dofhandler import start_assemble as _pattern
        return _pattern(N, f, symmetric)
    return Assembler(int(N))


def assemble_(a, edof, Ke, fe=None):
    """assemble!(a, edof, Ke) for an Assembler, assemble!(A, dofs, Ke[, fe]) for a pattern
    assembler, or assemble!(g, edof, ge) for a vector g."""
    from .dofhandler import AssemblerSparsityPattern, assemble_ as _pattern_assemble
    if isinstance(a, AssemblerSparsityPattern):
        return _pattern_assemble(a, edof, Ke, fe)
    edof = np.ascontiguousarray(edof, dtype=np.int64)
    if isinstance(a, Assembler):
        K = np.asfortranarray(Ke, dtype=np.float64)
        L.check(L.load().hdg_assembler_add(a._h, len(edof), L.i64ptr(edof), L.dptr(K)))
        return a
    g = a
    np.add.at(g, edof - 1, np.asarray(Ke, dtype=g.dtype))
    return g


def end_assemble(a: Assembler) -> SparseMatrixCSC:
    m, n, nnz = C.c_int64(), C.c_int64(), C.c_int64()
    L.check(L.load().hdg_assembler_finish(a._h, C.byref(m), C.byref(n), C.byref(nnz)))
    colptr = np.zeros(n.value + 1, np.int64)
    rowval = np.zeros(nnz.value, np.int64)
    nzval = np.zeros(nnz.value)
    L.check(L.load().hdg_assembler_get_csc(a._h, 1, L.i64ptr(colptr), L.i64ptr(rowval), L.dptr(nzval)))
    return SparseMatrixCSC(m.value, n.value, colptr, rowval, nzval)
