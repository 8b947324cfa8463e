"""The HDG Poisson flow of examples/poisson2D_HDG.jl on the GPU:

    K, b, K_e, b_e = doassemble(Vh, Wh, Mh, tau, f)       # :58-186 (device)
    apply_(K, b, dbc)                                      # apply!, src/boundary.jl:121-158
    uhat = solve(K, b)                                     # K \\ b, :195 (device CG)
    get_usigma_(sigma_h, u_h, uhat_h, uhat, K_e, b_e, mesh)  # get_uσ!, :197-212
    errornorm(u_h, u_ex)                                   # src/DiscreteFunctions.jl:97-120

K is a TraceSystem: the condensed global trace matrix and its right-hand side live on the
device; b, K_e and b_e are views of the same object.  Their values can be exported to the host
(TraceSystem.csc(), .element_blocks()) for inspection and parity checks.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .fields import as_field
from .spaces import ScalarFunctionSpace, ScalarTraceFunctionSpace, VectorFunctionSpace


class SolveStats:
    def __init__(self, s: L.hdg_stats):
        self.iterations = s.iterations
        self.outer = s.outer
        self.rel_residual = s.rel_residual
        self.converged = bool(s.converged)

    def __repr__(self):
        return (f"SolveStats(iterations={self.iterations}, outer={self.outer}, "
                f"rel_residual={self.rel_residual:.3e}, converged={self.converged})")


class TraceSystem:
    """Assembled + condensed HDG trace system on the device (hdg_system)."""

    def __init__(self, space_handle, tau=1.0, f=None, kappa=None, kappa_cell=None, precision=L.PREC_FP64,
                 he_tau=False):
        self.sp = space_handle
        self.ctx = space_handle.mesh.ctx
        self.precision = precision
        h = C.c_void_p()
        fc, kc, kcell = self._coef(f, kappa, kappa_cell)
        lib = L.load()
        if he_tau:  # the choice is taken by the system at creation; the shared space is reset
            L.check(lib.hdg_space_set_he_tau(self.sp.h, 1))
        try:
            L.check(lib.hdg_assemble_condense(self.sp.h, float(tau), fc, kc, kcell, int(precision), C.byref(h)),
                    self.ctx)
        finally:
            if he_tau:
                lib.hdg_space_set_he_tau(self.sp.h, 0)
        self._h = h
        nd, nnz, n, m = C.c_int(), C.c_int64(), C.c_int(), C.c_int()
        L.check(L.load().hdg_system_sizes(self._h, C.byref(nd), C.byref(nnz), C.byref(n), C.byref(m)))
        self.ndofs, self.nnz, self.n, self.m = nd.value, nnz.value, n.value, m.value
        self.ncells = space_handle.mesh.ncells
        self.stats = None

    def _coef(self, f, kappa, kappa_cell):
        f, kappa = as_field(f), as_field(kappa)
        self._keep = []
        fc = f.as_c() if f is not None else None
        kc = kappa.as_c() if kappa is not None else None
        self._keep += [fc, kc]
        kcell = None
        if kappa_cell is not None:
            kk = L.f64(kappa_cell)
            if kk.size != self.sp.mesh.ncells:
                raise ValueError("kappa_cell must have one value per cell")
            self._keep.append(kk)
            kcell = L.dptr(kk)
        return (C.byref(fc) if fc is not None else None, C.byref(kc) if kc is not None else None, kcell)

    @property
    def handle(self):
        return self._h

    def __del__(self):
        try:
            if self._h:
                L.load().hdg_system_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def reassemble(self, tau=1.0, f=None, kappa=None, kappa_cell=None, resident=False):
        """Assemble and condense again with new coefficients; resident=True reuses the ones already
        on the device (no host transfer)."""
        if resident:
            L.check(L.load().hdg_system_reassemble_resident(self._h), self.ctx)
            return
        fc, kc, kcell = self._coef(f, kappa, kappa_cell)
        L.check(L.load().hdg_system_reassemble(self._h, float(tau), fc, kc, kcell), self.ctx)

    # ---- exports ------------------------------------------------------------------------
    def csc(self, base: int = 0):
        """(colptr, rowval, nzval, rhs) of K and b as the reference holds them."""
        colptr = np.zeros(self.ndofs + 1, np.int64)
        rowval = np.zeros(self.nnz, np.int64)
        nzval = np.zeros(self.nnz)
        rhs = np.zeros(self.ndofs)
        L.check(L.load().hdg_system_get_csc(self._h, base, L.i64ptr(colptr), L.i64ptr(rowval), L.dptr(nzval),
                                            L.dptr(rhs)), self.ctx)
        return colptr, rowval, nzval, rhs

    def to_scipy(self):
        import scipy.sparse as sp
        colptr, rowval, nzval, rhs = self.csc(0)
        return sp.csc_matrix((nzval, rowval, colptr), shape=(self.ndofs, self.ndofs)), rhs

    def element_blocks(self):
        nc, n, m = self.ncells, self.n, self.m
        Ate, bte = np.zeros((nc, m, m)), np.zeros((nc, m))
        Ke, be = np.zeros((nc, n, m)), np.zeros((nc, n))
        L.check(L.load().hdg_system_get_element_blocks(self._h, L.dptr(Ate), L.dptr(bte), L.dptr(Ke), L.dptr(be)),
                self.ctx)
        return Ate, bte, Ke, be

    # ---- boundary conditions, solve, recovery ---------------------------------------------
    def apply_dirichlet(self, dofs, vals):
        d, v = L.i32(dofs), L.f64(vals)
        L.check(L.load().hdg_apply_dirichlet(self._h, L.i32ptr(d), L.dptr(v), len(d)), self.ctx)

    def solve(self, tol=1e-12, maxit=100000, precision=None, chunk=32, inner_tol=1e-5, to_host=True,
              preconditioner=L.PRECOND_JACOBI, refine=0, refine_tol=1e-6):
        """K \\ b by preconditioned CG (Jacobi, or the multigrid V-cycle with preconditioner=PRECOND_AMG).

        refine > 0 follows the CG with that many FP64 iterative-refinement steps on a
        double-double residual (hdg_refine), each correction solved to refine_tol; the result is
        then the assembled FP64 system's solution to a few ulps instead of the CG's tolerance."""
        o = L.hdg_solver(float(tol), int(maxit), int(self.precision if precision is None else precision), int(chunk),
                         float(inner_tol), int(preconditioner))
        st = L.hdg_stats()
        out = np.zeros(self.ndofs) if to_host else None
        L.check(L.load().hdg_solve(self._h, C.byref(o), None if refine else L.dptr(out), C.byref(st)), self.ctx)
        self.stats = SolveStats(st)
        if refine:
            rs = L.hdg_stats()
            L.check(L.load().hdg_refine(self._h, C.byref(o), int(refine), float(refine_tol), L.dptr(out),
                                        C.byref(rs)), self.ctx)
            self.refine_stats = SolveStats(rs)
        return out

    def recover(self, to_host=True):
        if not to_host:
            L.check(L.load().hdg_recover(self._h, None, None, None), self.ctx)
            return None
        nw = self.sp.nw
        q = np.zeros((self.ncells, 2 * nw))
        u = np.zeros((self.ncells, nw))
        uc = np.zeros((self.ncells, 3, self.sp.nt))
        L.check(L.load().hdg_recover(self._h, L.dptr(q), L.dptr(u), L.dptr(uc)), self.ctx)
        return q, u, uc

    def timings(self) -> dict:
        """Per-phase device times recorded while the context's profiling was on (ms)."""
        t = L.hdg_timings()
        L.check(L.load().hdg_system_timings(self._h, C.byref(t)), self.ctx)
        return {k: getattr(t, k) for k, _ in L.hdg_timings._fields_}

    def errornorm(self, u_ex) -> float:
        fc = as_field(u_ex).as_c()
        out = C.c_double()
        L.check(L.load().hdg_errornorm_l2sq(self._h, C.byref(fc), C.byref(out)), self.ctx)
        return out.value


class _RhsView:
    """b of doassemble: the right-hand side held by the TraceSystem."""

    def __init__(self, system):
        self.system = system

    def __array__(self, dtype=None, copy=None):
        return self.system.csc()[3]


class _LocalView:
    """K_e / b_e of doassemble: the condensed local operators held by the TraceSystem."""

    def __init__(self, system, which):
        self.system, self.which = system, which

    def __array__(self, dtype=None, copy=None):
        Ate, bte, Ke, be = self.system.element_blocks()
        return Ke if self.which == "K" else be


def doassemble(Vh: VectorFunctionSpace, Wh: ScalarFunctionSpace, Mh: ScalarTraceFunctionSpace, tau: float = 1.0,
               f=None, kappa=None, kappa_cell=None, precision=L.PREC_FP64, he_tau=False):
    """doassemble(Vh, Wh, Mh, τ) of examples/poisson2D_HDG.jl:58-186 on the device.
    Returns (K, b, K_e, b_e); K is the TraceSystem, the others are views of it.
    he_tau=True puts τ into He (the reference's He has none, :149; they agree for τ = 1)."""
    if not (Vh.sp is Wh.sp is Mh.sp):
        raise ValueError("Vh, Wh and Mh must be built on the same mesh with the same degree and quadrature")
    K = TraceSystem(Wh.sp, tau, f, kappa, kappa_cell, precision, he_tau)
    return K, _RhsView(K), _LocalView(K, "K"), _LocalView(K, "b")


class Dirichlet:
    """Dirichlet(û_h, mesh, faceset, g) on the trace space (src/boundary.jl:11-42), or
    Dirichlet(u, dh, faceset, g) on a nodal field of a DofHandler (src/boundary.jl:44-95)."""

    def __init__(self, u, mesh, faceset: str, g=None, projection: str = "reference"):
        """projection="l2" takes the L2 projection of g onto the trace basis (hdg_dirichlet_l2)
        instead of the reference's accumulation (src/boundary.jl:27-37)."""
        from .dofhandler import DofHandler, DirichletDH
        if isinstance(mesh, DofHandler):
            d = DirichletDH(u, mesh, faceset, g if g is not None else (lambda x: 0.0))
            self.prescribed_dofs, self.values = d.prescribed_dofs, d.values
            return
        fs = u.fs if isinstance(u, TrialFunction) else u
        if not isinstance(fs, ScalarTraceFunctionSpace):
            raise NotImplementedError("the HDG path prescribes trace dofs (ScalarTraceFunctionSpace)")
        g = as_field(g if g is not None else 0.0)
        gc = g.as_c()
        n = C.c_int()
        if projection not in ("reference", "l2"):
            raise ValueError("projection is 'reference' or 'l2'")
        fn = L.load().hdg_dirichlet_l2 if projection == "l2" else L.load().hdg_dirichlet
        L.check(fn(fs.sp.h, faceset.encode(), C.byref(gc), None, None, C.byref(n)), mesh.ctx)
        self.prescribed_dofs = np.zeros(n.value, np.int32)
        self.values = np.zeros(n.value)
        L.check(fn(fs.sp.h, faceset.encode(), C.byref(gc), L.i32ptr(self.prescribed_dofs), L.dptr(self.values),
                   C.byref(n)), mesh.ctx)


def apply_(K, b, dbc: Dirichlet):
    """apply!(K, b, dbc) (src/boundary.jl:121-158, :121-158) on the device system: the HDG
    TraceSystem of doassemble or the LagrangeSystem of doassemble_cg (b is refreshed in place)."""
    from .lagrange import LagrangeSystem
    if isinstance(K, LagrangeSystem):
        K.apply_dirichlet(dbc.prescribed_dofs, dbc.values)
        if b is not None and b is not K.b:
            b[:] = K.b
        return
    if not isinstance(K, TraceSystem):
        raise TypeError("apply_ works on the system returned by doassemble or doassemble_cg")
    K.apply_dirichlet(dbc.prescribed_dofs, dbc.values)


def solve(K, b=None, **opts) -> np.ndarray:
    """û = K \\ b (examples/poisson2D_HDG.jl:195, poisson2D_CG.jl:126): PCG on the device."""
    return K.solve(**opts)


class TrialFunction:
    """TrialFunction(fs): m_values[cell, i] (or [cell, i, face] on the trace) (src/DiscreteFunctions.jl:27-54)."""

    def __init__(self, fs):
        self.fs = fs
        nc = fs.mesh.ncells
        if isinstance(fs, ScalarTraceFunctionSpace):
            self.m_values = np.full((nc, fs.getnbasefunctions(), 3), np.nan)
        else:
            self.m_values = np.full((nc, fs.getnbasefunctions()), np.nan)
        self.system = None

    def getnbasefunctions(self):
        return self.fs.getnbasefunctions()


def get_usigma_(sigma_h: TrialFunction, u_h: TrialFunction, uhat_h: TrialFunction, uhat, K_e, b_e, mesh):
    """get_uσ! (examples/poisson2D_HDG.jl:197-212): recover q and u cell by cell on the device."""
    K = K_e.system if isinstance(K_e, _LocalView) else K_e
    q, u, uc = K.recover()
    sigma_h.m_values[:] = q
    u_h.m_values[:] = u
    uhat_h.m_values[:] = np.transpose(uc, (0, 2, 1))
    u_h.system = sigma_h.system = uhat_h.system = K


def nodal_avg(u_h: TrialFunction) -> np.ndarray:
    """nodal_avg(u_h) (src/DiscreteFunctions.jl:81-95): per mesh node, the mean of the recovered u
    over the node's cells, evaluated at the node."""
    K = u_h.system
    if K is None:
        raise ValueError("u_h has no recovered values (call get_usigma_ first)")
    out = np.zeros(K.sp.mesh.nnodes)
    L.check(L.load().hdg_nodal_avg(K._h, L.dptr(out)), K.ctx)
    return out


def errornorm(u_h: TrialFunction, u_ex, norm_type: str = "L2") -> float:
    """errornorm(u_h, u_ex): the SQUARED L2 error (src/DiscreteFunctions.jl:97-120), on the device."""
    if norm_type != "L2":
        raise ValueError(f"Norm {norm_type} not available")
    if u_h.system is None:
        raise ValueError("u_h has no recovered values (call get_usigma_ or reconstruct_ first)")
    from .lagrange import LagrangeSystem
    if isinstance(u_h.system, LagrangeSystem):
        return u_h.system.errornorm(u_h.dof_values, u_ex)
    return u_h.system.errornorm(u_ex)


class CellIterator:
    """CellIterator(mesh) (src/iterator.jl:10-65): yields itself with current_cellid, nodes, coords."""

    def __init__(self, mesh):
        self.mesh = mesh
        self.current_cellid = 0
        self.nodes = (0, 0, 0)
        self.coords = []

    def __iter__(self):
        cells = self.mesh._topology()[1]
        xy = self.mesh._topology()[0]
        for c in range(self.mesh.ncells):
            self.current_cellid = c + 1
            self.nodes = tuple(int(v) for v in cells[c])
            self.coords = [tuple(xy[n - 1]) for n in self.nodes]
            yield self

    def __len__(self):
        return self.mesh.ncells


def solve_poisson(mesh, p: int, f, tau: float = 1.0, kappa=None, kappa_cell=None, faceset="boundary", g=None,
                  quad_degree=None, precision=L.PREC_FP64, tol=1e-12, maxit=100000, preconditioner=L.PRECOND_JACOBI):
    """The whole poisson2D_HDG flow in one C-ABI call (hdg_solve_poisson); returns (uhat, q, u, stats)."""
    from .spaces import GenericFiniteElement, Dubiner, _handle
    sp = _handle(mesh, p, quad_degree if quad_degree is not None else p + 1)
    f, kappa, g = as_field(f), as_field(kappa), as_field(g if g is not None else 0.0)
    fc, gc = f.as_c(), g.as_c()
    kc = kappa.as_c() if kappa is not None else None
    kk = L.f64(kappa_cell) if kappa_cell is not None else None
    o = L.hdg_solver(float(tol), int(maxit), int(precision), 32, 1e-5, int(preconditioner))
    st = L.hdg_stats()
    nd = mesh.nfaces * sp.nt
    uhat, q, u = np.zeros(nd), np.zeros((mesh.ncells, sp.nv)), np.zeros((mesh.ncells, sp.nw))
    L.check(L.load().hdg_solve_poisson(sp.h, float(tau), C.byref(fc), C.byref(kc) if kc is not None else None,
                                       L.dptr(kk), faceset.encode(), C.byref(gc), C.byref(o), L.dptr(uhat), L.dptr(q),
                                       L.dptr(u), C.byref(st)), mesh.ctx)
    return uhat, q, u, SolveStats(st)
