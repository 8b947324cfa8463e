"""hdgref — Python side of the CPU oracle for the HDG Poisson flow.

TEST INFRASTRUCTURE ONLY.  Loaded by tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline leg as the test oracle; the product never imports it.

The C++ half (``hdgref.cpp``) restates the reference's element loop, condensation and
assembly; this half restates the Triangle-format reader (src/triangle_mesh.jl:1-126) and
performs the global solve ``K \\ b`` (examples/poisson2D_HDG.jl:195) with scipy's SuperLU,
standing in for the UMFPACK LU that Julia's SparseArrays uses for a non-Hermitian matrix.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libhdgref.so")
_lock = threading.Lock()
_lib = None

# field kinds shared with the GPU library (hdg.h: HDG_FIELD_*)
F_CONST, F_SINSIN, F_BUMPS, F_FOURIER, F_EXP_FOURIER = 0, 1, 2, 3, 4


def build(force: bool = False) -> str:
    """Compile the oracle's C++ half into oracle/_build/libhdgref.so."""
    os.makedirs(os.path.dirname(_SO), exist_ok=True)
    src = os.path.join(_HERE, "hdgref.cpp")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _SO


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_SO)
            vp, ip, dp, i64p = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_int64)
            L.hr_rect_mesh.restype = vp
            L.hr_rect_mesh.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]
            L.hr_mesh_from_triangle.restype = vp
            L.hr_mesh_from_triangle.argtypes = [C.c_int, dp, C.c_int, ip, C.c_int, ip]
            L.hr_mesh_free.argtypes = [vp]
            L.hr_mesh_sizes.argtypes = [vp, ip, ip, ip]
            L.hr_mesh_arrays.argtypes = [vp, dp, ip, ip, ip]
            L.hr_mesh_set_xy.argtypes = [vp, dp]
            L.hr_mesh_faceset.argtypes = [vp, C.c_char_p, ip]
            L.hr_table_sizes.argtypes = [C.c_int, C.c_int, ip, ip]
            L.hr_tables.argtypes = [C.c_int, C.c_int] + [dp] * 9
            L.hr_dubiner.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, dp, dp, dp]
            L.hr_legendre.restype = C.c_double
            L.hr_legendre.argtypes = [C.c_int, C.c_double]
            L.hr_rule.argtypes = [C.c_int, C.c_int, dp, dp, dp]
            L.hr_cell_geometry.argtypes = [vp, C.c_int, dp, dp, dp, dp]
            L.hr_element_blocks.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, dp] + [dp] * 7
            L.hr_assemble.restype = vp
            L.hr_assemble.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, dp, C.c_int, C.c_int, dp,
                                      dp, C.c_int, ip]
            L.hr_assemble_ex.restype = vp
            L.hr_assemble_ex.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, dp, C.c_int, C.c_int,
                                         dp, dp, C.c_int, C.c_int, ip]
            L.hr_dirichlet_l2.argtypes = [vp, C.c_int, C.c_int, C.c_char_p, C.c_int, C.c_int, dp, ip, dp]
            L.hr_system_free.argtypes = [vp]
            L.hr_system_sizes.argtypes = [vp, ip, i64p, ip, ip]
            L.hr_system_csc.argtypes = [vp, i64p, i64p, dp, dp]
            L.hr_system_set_csc_values.argtypes = [vp, dp, dp]
            L.hr_system_local.argtypes = [vp, dp, dp]
            L.hr_dirichlet.argtypes = [vp, C.c_int, C.c_int, C.c_char_p, C.c_int, C.c_int, dp, ip, dp]
            L.hr_apply.argtypes = [vp, C.c_int, ip, dp]
            L.hr_recover.argtypes = [vp, dp, dp, dp, dp]
            L.hr_errornorm.restype = C.c_double
            L.hr_errornorm.argtypes = [vp, C.c_int, C.c_int, dp, C.c_int, C.c_int, dp]
            L.hr_eval_field.restype = C.c_double
            L.hr_eval_field.argtypes = [C.c_int, C.c_int, dp, C.c_double, C.c_double]
            L.hr_csc_residual_dd.argtypes = [C.c_int, i64p, i64p, dp, dp, dp, dp]
            _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int)) if a is not None else None


def _i64p(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64)) if a is not None else None


def _field(spec):
    kind, prm = spec if spec is not None else (F_CONST, [0.0])
    prm = np.ascontiguousarray(prm, dtype=np.float64).ravel()
    if prm.size == 0:
        prm = np.zeros(1)
    return int(kind), prm


class Mesh:
    """Oracle mesh (1-based ids, as in the reference's PolygonalMesh, src/mesh.jl:43-49)."""

    def __init__(self, handle):
        if not handle:
            raise ValueError("mesh construction failed")
        self.h = handle
        L = lib()
        nn, nc, nf = C.c_int(), C.c_int(), C.c_int()
        L.hr_mesh_sizes(self.h, C.byref(nn), C.byref(nc), C.byref(nf))
        self.nnodes, self.ncells, self.nfaces = nn.value, nc.value, nf.value
        self.xy = np.zeros((self.nnodes, 2))
        self.cells = np.zeros((self.ncells, 3), np.int32)
        self.cell_faces = np.zeros((self.ncells, 3), np.int32)
        self.faces = np.zeros((self.nfaces, 4), np.int32)
        L.hr_mesh_arrays(self.h, _dp(self.xy), _ip(self.cells), _ip(self.cell_faces), _ip(self.faces))

    def __del__(self):
        try:
            lib().hr_mesh_free(self.h)
        except Exception:
            pass

    def faceset(self, name: str) -> np.ndarray:
        n = lib().hr_mesh_faceset(self.h, name.encode(), None)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(max(n, 1), np.int32)
        lib().hr_mesh_faceset(self.h, name.encode(), _ip(out))
        return out[:n]

    def set_xy(self, xy):
        xy = np.ascontiguousarray(xy, dtype=np.float64)
        lib().hr_mesh_set_xy(self.h, _dp(xy))
        self.xy = xy.copy()

    def orientation(self, c: int, f: int) -> bool:
        """face_orientation(mesh, c, f) for 0-based c, f (src/mesh.jl:51-54)."""
        k = ((1, 2), (2, 0), (0, 1))[f]
        return bool(self.cells[c, k[1]] > self.cells[c, k[0]])

    def cell_geometry(self, c: int):
        detJ = C.c_double()
        Jinv = np.zeros(4)
        detJf = np.zeros(3)
        nrm = np.zeros(6)
        rc = lib().hr_cell_geometry(self.h, c, C.byref(detJ), _dp(Jinv), _dp(detJf), _dp(nrm))
        if rc != 0:
            raise ValueError("det(J) is not positive")
        return detJ.value, Jinv.reshape(2, 2), detJf, nrm.reshape(3, 2)


def rectangle_mesh(nx: int, ny: int, LL=(0.0, 0.0), UR=(1.0, 1.0)) -> Mesh:
    return Mesh(lib().hr_rect_mesh(nx, ny, LL[0], LL[1], UR[0], UR[1]))


_NUM = re.compile(r"\b((\d*\.)?\d+)\b")


def _read_line(ln, types):
    # read_line, src/triangle_mesh.jl:2-5 (unsigned numbers only, as in the reference)
    return [t(m.group(0)) for t, m in zip(types, _NUM.finditer(ln))]


def _records(path):
    first = True
    for ln in open(path):
        if re.match(r"^\s*(?:#|$)", ln):
            continue
        if first:
            first = False
            continue
        yield ln


def parse_mesh_triangle(root: str) -> Mesh:
    """parse_mesh_triangle(root_file), src/triangle_mesh.jl:115-126."""
    nodes = [_read_line(ln, (int, float, float, int))[1:3] for ln in _records(root + ".node")]
    edges = [_read_line(ln, (int, int, int, int))[1:4] for ln in _records(root + ".edge")]
    cells = [_read_line(ln, (int, int, int, int))[1:4] for ln in _records(root + ".ele")]
    xy = np.ascontiguousarray(nodes, dtype=np.float64)
    ele = np.ascontiguousarray(cells, dtype=np.int32)
    ed = np.ascontiguousarray(edges, dtype=np.int32)
    return Mesh(lib().hr_mesh_from_triangle(len(xy), _dp(xy), len(ele), _ip(ele), len(ed), _ip(ed)))


def tables(p: int, qd: int | None = None):
    qd = p + 1 if qd is None else qd
    nq, nfq = C.c_int(), C.c_int()
    if lib().hr_table_sizes(p, qd, C.byref(nq), C.byref(nfq)) != 0:
        raise ValueError(f"Quadrature rule of order {qd} not available")
    nq, nfq = nq.value, nfq.value
    nw, nt = (p + 1) * (p + 2) // 2, p + 1
    out = dict(vx=np.zeros(nq), vy=np.zeros(nq), vw=np.zeros(nq), N=np.zeros((nw, nq)), dN=np.zeros((nw, nq, 2)),
               fx=np.zeros(nfq), fw=np.zeros(nfq), E=np.zeros((nw, nfq, 3)), T=np.zeros((nt, nfq)))
    lib().hr_tables(p, qd, *[_dp(out[k]) for k in ("vx", "vy", "vw", "N", "dN", "fx", "fw", "E", "T")])
    return out


def rule(kind: int, order: int):
    n = lib().hr_rule(kind, order, None, None, None)
    if n < 0:
        raise ValueError("rule not available")
    x, y, w = np.zeros(n), np.zeros(n), np.zeros(n)
    lib().hr_rule(kind, order, _dp(x), _dp(y), _dp(w))
    return x, y, w


def dubiner(j, x, y, generic=False):
    v, gx, gy = C.c_double(), C.c_double(), C.c_double()
    lib().hr_dubiner(j, x, y, int(generic), C.byref(v), C.byref(gx), C.byref(gy))
    return v.value, np.array([gx.value, gy.value])


def element_blocks(mesh: Mesh, c: int, p: int, qd=None, tau=1.0, f=None):
    qd = p + 1 if qd is None else qd
    nw, nt = (p + 1) * (p + 2) // 2, p + 1
    nv, m = 2 * nw, 3 * nt
    fk, fp = _field(f)
    A, B, Cc = np.zeros((nv, nv)), np.zeros((nv, nw)), np.zeros((nw, nw))
    E, F, H, be = np.zeros((nv, m)), np.zeros((nw, m)), np.zeros((m, m)), np.zeros(nw)
    rc = lib().hr_element_blocks(mesh.h, c, p, qd, tau, fk, fp.size, _dp(fp), _dp(A), _dp(B), _dp(Cc), _dp(E),
                                 _dp(F), _dp(H), _dp(be))
    if rc != 0:
        raise ValueError(f"element_blocks failed ({rc})")
    return dict(A=A, B=B, C=Cc, E=E, F=F, H=H, be=be)


class System:
    """Assembled (condensed) trace system of the oracle: CSC K, rhs b, local K_e, b_e."""

    def __init__(self, mesh: Mesh, p: int, qd=None, tau=1.0, f=None, kappa=None, kappa_cell=None, threads=1,
                 he_tau=False):
        self.mesh, self.p = mesh, p
        self.qd = p + 1 if qd is None else qd
        fk, fp = _field(f)
        if kappa is not None:
            kk, kp = _field(kappa)
        else:
            kk, kp = -1, np.zeros(1)
        kc = None if kappa_cell is None else np.ascontiguousarray(kappa_cell, dtype=np.float64)
        st = C.c_int()
        self.h = lib().hr_assemble_ex(mesh.h, p, self.qd, tau, fk, fp.size, _dp(fp), kk, kp.size, _dp(kp), _dp(kc),
                                      threads, 1 if he_tau else 0, C.byref(st))
        if not self.h:
            raise ValueError(f"oracle assembly failed ({st.value})")
        nd, nnz, n, m = C.c_int(), C.c_int64(), C.c_int(), C.c_int()
        lib().hr_system_sizes(self.h, C.byref(nd), C.byref(nnz), C.byref(n), C.byref(m))
        self.ndofs, self.nnz, self.n, self.m = nd.value, nnz.value, n.value, m.value
        self.nt, self.nw = p + 1, (p + 1) * (p + 2) // 2

    def __del__(self):
        try:
            lib().hr_system_free(self.h)
        except Exception:
            pass

    def csc(self):
        import scipy.sparse as sp
        colptr = np.zeros(self.ndofs + 1, np.int64)
        rowval = np.zeros(self.nnz, np.int64)
        nzval = np.zeros(self.nnz)
        rhs = np.zeros(self.ndofs)
        lib().hr_system_csc(self.h, _i64p(colptr), _i64p(rowval), _dp(nzval), _dp(rhs))
        K = sp.csc_matrix((nzval, rowval, colptr), shape=(self.ndofs, self.ndofs))
        return K, rhs

    def local(self):
        nc = self.mesh.ncells
        Ke = np.zeros((nc, self.n, self.m))
        be = np.zeros((nc, self.n))
        lib().hr_system_local(self.h, _dp(Ke), _dp(be))
        return Ke, be

    def dirichlet(self, faceset="boundary", g=None, projection="reference"):
        """Trace Dirichlet dofs and values: the reference's accumulation, or (projection="l2") the
        L2 projection of g onto the trace basis."""
        gk, gp = _field(g)
        n = len(self.mesh.faceset(faceset)) * self.nt
        dofs = np.zeros(max(n, 1), np.int32)
        vals = np.zeros(max(n, 1))
        fn = lib().hr_dirichlet_l2 if projection == "l2" else lib().hr_dirichlet
        k = fn(self.mesh.h, self.p, self.qd, faceset.encode(), gk, gp.size, _dp(gp), _ip(dofs), _dp(vals))
        if k < 0:
            raise ValueError(f"Dirichlet failed ({k})")
        return dofs[:k], vals[:k]

    def apply(self, dofs, vals):
        dofs = np.ascontiguousarray(dofs, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        lib().hr_apply(self.h, len(dofs), _ip(dofs), _dp(vals))

    def solve(self, refine: int = 0):
        """û = K \\ b with SuperLU (examples/poisson2D_HDG.jl:195).  Julia's `\\` on a
        non-Hermitian SparseMatrixCSC calls UMFPACK, whose symmetric strategy (chosen for a matrix
        with a symmetric pattern and a zero-free diagonal, as K is) orders A'+A by minimum degree
        and prefers diagonal pivots with a relative tolerance of 0.001.  SuperLU is set up the
        same way: minimum degree on A'+A and diag_pivot_thresh = 0.001.

        refine > 0 adds up to that many steps of iterative refinement with the double-double
        residual (csc_residual_dd) and the same LU factors.  The direct solve alone carries a
        forward error of order cond(K) * 2^-53 (about 1e-12 on the 2*256^2-cell system); the
        refined solution is the assembled FP64 system's solution to about 1e-16, which is what
        a 1e-12 comparison of two solvers needs."""
        import scipy.sparse.linalg as spla
        K, b = self.csc()
        lu = spla.splu(K.tocsc(), permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.001)
        x = lu.solve(b)
        for _ in range(refine):
            d = lu.solve(csc_residual_dd(K, x, b))
            x = x + d
            if np.linalg.norm(d) <= 1e-17 * np.linalg.norm(x):
                break
        return x

    def recover(self, uhat):
        nc = self.mesh.ncells
        uhat = np.ascontiguousarray(uhat, dtype=np.float64)
        q = np.zeros((nc, 2 * self.nw))
        u = np.zeros((nc, self.nw))
        uc = np.zeros((nc, 3, self.nt))
        lib().hr_recover(self.h, _dp(uhat), _dp(q), _dp(u), _dp(uc))
        return q, u, uc


def errornorm(mesh: Mesh, p: int, u, u_ex, qd=None) -> float:
    """errornorm(u_h, u_ex): the squared L2 error (src/DiscreteFunctions.jl:97-120)."""
    qd = p + 1 if qd is None else qd
    uk, up = _field(u_ex)
    u = np.ascontiguousarray(u, dtype=np.float64)
    return lib().hr_errornorm(mesh.h, p, qd, _dp(u), uk, up.size, _dp(up))


def csc_residual_dd(K, x, b) -> np.ndarray:
    """b - K x for a scipy CSC matrix, summed in double-double arithmetic and rounded once
    (hr_csc_residual_dd)."""
    K = K.tocsc()
    colptr = np.ascontiguousarray(K.indptr, dtype=np.int64)
    rowval = np.ascontiguousarray(K.indices, dtype=np.int64)
    val = np.ascontiguousarray(K.data, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    r = np.zeros(K.shape[0])
    lib().hr_csc_residual_dd(K.shape[0], _i64p(colptr), _i64p(rowval), _dp(val), _dp(x), _dp(b), _dp(r))
    return r


def eval_field(spec, x, y) -> float:
    k, prm = _field(spec)
    return lib().hr_eval_field(k, prm.size, _dp(prm), float(x), float(y))


MANUFACTURED_F = (F_SINSIN, [2 * np.pi ** 2, 1.0, 1.0])
MANUFACTURED_U = (F_SINSIN, [1.0, 1.0, 1.0])


def solve_poisson(mesh: Mesh, p: int, qd=None, tau=1.0, f=MANUFACTURED_F, g=None, kappa=None, kappa_cell=None,
                  faceset="boundary", threads=1):
    """The whole poisson2D_HDG flow (examples/poisson2D_HDG.jl:58-218) on the oracle."""
    S = System(mesh, p, qd, tau, f, kappa, kappa_cell, threads)
    dofs, vals = S.dirichlet(faceset, g)
    S.apply(dofs, vals)
    uhat = S.solve()
    q, u, uc = S.recover(uhat)
    return dict(system=S, uhat=uhat, q=q, u=u, uhat_cell=uc, dofs=dofs, vals=vals)
