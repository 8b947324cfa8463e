"""The continuous-Galerkin Poisson path of examples/poisson2D_CG.jl on the device (csrc/lagrange.cu).

    Wh = ScalarFunctionSpace(mesh, ContinuousLagrange(2, RefTetrahedron, 1), update_face_data=False)
    u_h = TrialFunction(Wh)
    dh = DofHandler([u_h], mesh)
    K = create_sparsity_pattern(dh)
    dbc = Dirichlet(u_h, dh, "boundary", lambda x: 0.0)
    K, b = doassemble_cg(Wh, K, dh, f)        # the example's element loop + assemble!, on the device
    apply_(K, b, dbc)
    u = solve(K, b)
    reconstruct_(u_h, u, dh)
    errornorm(u_h, u_ex)                       # squared L2, <= 2e-4 on 10 x 10 (test_CGExample.jl:92)

`K` is a LagrangeSystem: the device copy of the caller's CSC pattern with its values; `K.csc()`
returns them as a scipy matrix, `b` is refreshed on the host after each device step."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .fields import as_field
from .spaces import ContinuousLagrange


class LagrangeSystem:
    """K and b of the CG Poisson problem on the device, in the DofHandler's CSC pattern."""

    def __init__(self, Wh, pattern, dh):
        fe = Wh.fe
        if not isinstance(fe, ContinuousLagrange):
            raise TypeError("doassemble_cg needs a ContinuousLagrange space")
        if dh.nvariables() != 1:
            raise NotImplementedError("doassemble_cg assembles one-field DofHandlers")
        mesh = Wh.mesh
        if mesh.ctx is None:
            raise ValueError("doassemble_cg needs a mesh on the device (built with a context)")
        self.ctx = mesh.ctx  # context handle
        self.mesh, self.dh = mesh, dh
        self.pattern = pattern.tocsc()
        self.pattern.sort_indices()
        self.ndofs = dh.ndofs()
        nl = fe.getnbasefunctions()
        if dh.cell_dofs.size != mesh.ncells * nl:
            # src/dofhandler.jl:118-122 pushes one dof when it meets an entity with several dofs a
            # second time, so from order 3 on the cells do not hold a full set of dofs
            raise NotImplementedError("the DofHandler numbering of this order does not give every cell "
                                      f"{nl} dofs (orders 1 and 2 do)")
        cd = np.ascontiguousarray(dh.cell_dofs.reshape(mesh.ncells, nl), dtype=np.int32)
        colptr = np.ascontiguousarray(self.pattern.indptr, dtype=np.int64)
        rowval = np.ascontiguousarray(self.pattern.indices, dtype=np.int64)
        h = C.c_void_p()
        L.check(L.load().hdg_lagrange_create(self.ctx, mesh.handle, int(fe.order), int(Wh.quad_degree),
                                             int(self.ndofs), L.i32ptr(cd), int(rowval.size), L.i64ptr(colptr),
                                             L.i64ptr(rowval), C.byref(h)), self.ctx)
        self.h = h
        self.nnz = int(rowval.size)
        self.b = np.zeros(self.ndofs)
        self.u = None
        self.stats = None

    def assemble(self, f, kappa_cell=None):
        fc = as_field(f).as_c()
        kc = None if kappa_cell is None else np.ascontiguousarray(kappa_cell, dtype=np.float64)
        L.check(L.load().hdg_lagrange_assemble(self.h, C.byref(fc), L.dptr(kc)), self.ctx)
        self._refresh_b()

    def _refresh_b(self):
        L.check(L.load().hdg_lagrange_get_csc(self.h, None, L.dptr(self.b)), self.ctx)

    def csc(self):
        """K as a scipy CSC matrix (the stored values of the pattern)."""
        import scipy.sparse as sp
        v = np.zeros(self.nnz)
        L.check(L.load().hdg_lagrange_get_csc(self.h, L.dptr(v), None), self.ctx)
        return sp.csc_matrix((v, self.pattern.indices, self.pattern.indptr), shape=self.pattern.shape)

    def apply_dirichlet(self, dofs, vals):
        d = np.ascontiguousarray(dofs, dtype=np.int32)
        v = np.ascontiguousarray(vals, dtype=np.float64)
        L.check(L.load().hdg_lagrange_apply_dirichlet(self.h, L.i32ptr(d), L.dptr(v), int(d.size)), self.ctx)
        self._refresh_b()

    def solve(self, tol=1e-12, maxit=100000):
        o = L.hdg_solver(float(tol), int(maxit), int(L.PREC_FP64), 32, 1e-5, int(L.PRECOND_JACOBI))
        st = L.hdg_stats()
        u = np.zeros(self.ndofs)
        L.check(L.load().hdg_lagrange_solve(self.h, C.byref(o), L.dptr(u), C.byref(st)), self.ctx)
        from .system import SolveStats
        self.stats = SolveStats(st)
        self.u = u
        return u

    def errornorm(self, u, u_ex):
        out = C.c_double()
        ue = as_field(u_ex).as_c()
        uu = np.ascontiguousarray(u, dtype=np.float64)
        L.check(L.load().hdg_lagrange_errornorm_l2sq(self.h, L.dptr(uu), C.byref(ue), C.byref(out)), self.ctx)
        return out.value

    def __del__(self):
        try:
            if self.h:
                L.load().hdg_lagrange_destroy(self.h)
                self.h = None
        except Exception:
            pass


def doassemble_cg(Wh, K, dh, f, kappa_cell=None):
    """doassemble(Wh, K, dh) of examples/poisson2D_CG.jl:69-116 on the device: the element loop
    (stiffness int grad v . grad u, load int f v) and assemble! into the stored entries of K.
    Returns (LagrangeSystem, b)."""
    S = LagrangeSystem(Wh, K, dh)
    S.assemble(f, kappa_cell)
    dh._lagrange_system = S  # reconstruct_ hands it to u_h, so that errornorm finds the tables
    return S, S.b


def reconstruct_(u_h, u, dh):
    """reconstruct!(u_h, u, dh) (src/dofhandler.jl:223-229): per cell, the values of its dofs."""
    nl = u_h.getnbasefunctions()
    cd = dh.cell_dofs.reshape(-1, nl) - 1
    u_h.m_values[:] = np.asarray(u)[cd]
    u_h.dof_values = np.asarray(u, dtype=np.float64)
    u_h.system = getattr(dh, "_lagrange_system", None)
    return u_h
