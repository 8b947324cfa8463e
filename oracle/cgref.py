"""cgref — CPU oracle of the continuous-Galerkin Poisson example (examples/poisson2D_CG.jl).

TEST INFRASTRUCTURE ONLY.  Loaded by tests/ and bench.py's CPU-baseline leg as the test oracle;
the product never imports it.

A numpy/scipy restatement, for meshes the oracle finishes in seconds:
  * dof numbering of a one-field DofHandler (src/dofhandler.jl:88-149): cells in order; the
    cell's vertices, then (order 2) its faces in local order, each new entity getting the next
    dof, a seen one its recorded dof;
  * the nodal basis of ContinuousLagrange{2,RefTetrahedron,k} (src/LagrangeFE.jl:17-39) from a
    monomial Vandermonde matrix at the nodal points of src/shapes.jl:46-77 (the library builds it
    from the Dubiner basis instead: the two must agree);
  * the element loop of doassemble (poisson2D_CG.jl:76-113) with the oracle's quadrature rules
    (hdgref), COO -> CSC summation, apply! (src/boundary.jl:121-158), K \\ b with SuperLU, and
    errornorm (src/DiscreteFunctions.jl:97-120).
Pinned by the reference's own bound: errornorm <= 2e-4 on the 10 x 10 P1 example
(test/test_CGExample.jl:92-93, examples/poisson2D_CG.jl:139-140).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import hdgref

EDGES = (((1.0, 0.0), (0.0, 1.0)), ((0.0, 1.0), (0.0, 0.0)), ((0.0, 0.0), (1.0, 0.0)))


def nodal_points(k: int) -> np.ndarray:
    pts = [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0)]
    for a, b in EDGES:
        for i in range(1, k):
            pts.append((a[0] + i * (b[0] - a[0]) / k, a[1] + i * (b[1] - a[1]) / k))
    for i in range(1, k):
        for j in range(1, k - i):
            pts.append((j / k, i / k))
    return np.array(pts)


def _monomials(k, x, y):
    """values and gradients of x^a y^b, a + b <= k, at the points (x, y)."""
    v, gx, gy = [], [], []
    for n in range(k + 1):
        for b in range(n + 1):
            a = n - b
            v.append(x ** a * y ** b)
            gx.append(a * x ** max(a - 1, 0) * y ** b if a > 0 else 0.0 * x)
            gy.append(b * x ** a * y ** max(b - 1, 0) if b > 0 else 0.0 * y)
    return np.array(v), np.array(gx), np.array(gy)


def lagrange_tables(k: int, x, y):
    """N [nl][nq] and reference gradients dN [nl][nq][2] of the nodal basis at (x, y)."""
    P = nodal_points(k)
    V = _monomials(k, P[:, 0], P[:, 1])[0].T       # V[i][j] = m_j(node_i)
    Cm = np.linalg.inv(V)                           # phi_k = sum_j C[j][k] m_j
    m, mx, my = _monomials(k, np.asarray(x, float), np.asarray(y, float))
    N = Cm.T @ m
    dN = np.stack([Cm.T @ mx, Cm.T @ my], axis=-1)
    return N, dN


def distribute_dofs(mesh: "hdgref.Mesh", k: int) -> np.ndarray:
    """cell_dofs (ncells x nl, 1-based) of a one-field DofHandler of order 1 or 2."""
    if k not in (1, 2):
        raise ValueError("the oracle numbers orders 1 and 2")
    vd, fd = {}, {}
    nxt = 1
    rows = []
    for c in range(mesh.ncells):
        row = []
        ents = [(vd, int(v)) for v in mesh.cells[c]]
        if k == 2:
            ents += [(fd, int(f)) for f in mesh.cell_faces[c]]
        for d, key in ents:
            if key not in d:
                d[key] = nxt
                nxt += 1
            row.append(d[key])
        rows.append(row)
    return np.array(rows, dtype=np.int64)


def assemble(mesh, k: int, f, qd: int | None = None, kappa_cell=None, cell_dofs=None):
    """(K CSC, b, cell_dofs) of doassemble; f is an hdgref field spec (x, y) -> value."""
    qd = k + 1 if qd is None else qd
    t = hdgref.tables(1, qd)
    qx, qy, qw = t["vx"], t["vy"], t["vw"]
    N, dN = lagrange_tables(k, qx, qy)
    cd = distribute_dofs(mesh, k) if cell_dofs is None else np.asarray(cell_dofs)
    nd = int(cd.max())
    nl = N.shape[0]
    I, J, V = [], [], []
    b = np.zeros(nd)
    for c in range(mesh.ncells):
        v = mesh.xy[mesh.cells[c] - 1]
        Jm = np.array([[v[1, 0] - v[0, 0], v[2, 0] - v[0, 0]], [v[1, 1] - v[0, 1], v[2, 1] - v[0, 1]]])
        detJ = Jm[0, 0] * Jm[1, 1] - Jm[0, 1] * Jm[1, 0]
        if not detJ > 0:
            raise ValueError("det(J) is not positive")
        Ji = np.linalg.inv(Jm)
        kc = 1.0 if kappa_cell is None else float(kappa_cell[c])
        Ke = np.zeros((nl, nl))
        fe = np.zeros(nl)
        for q in range(len(qw)):
            dV = detJ * qw[q]
            g = dN[:, q, :] @ Ji                   # dNdx = dNdxi . Jinv
            Ke += kc * (g @ g.T) * dV
            xq = (1 - qx[q] - qy[q]) * v[0] + qx[q] * v[1] + qy[q] * v[2]
            fe += hdgref.eval_field(f, xq[0], xq[1]) * N[:, q] * dV
        dofs = cd[c] - 1
        I.extend(np.repeat(dofs, nl))
        J.extend(np.tile(dofs, nl))
        V.extend(Ke.ravel())
        np.add.at(b, dofs, fe)
    K = sp.csc_matrix((V, (I, J)), shape=(nd, nd))
    K.sum_duplicates()
    K.sort_indices()
    return K, b, cd


def apply_dirichlet(K, b, dofs, vals):
    """apply!(K, b, dbc), APPLY_TRANSPOSE (src/boundary.jl:121-158); dofs 1-based."""
    K = K.tocsc(copy=True)
    b = b.copy()
    n = K.shape[0]
    m = sum(abs(K[i, i]) for i in range(n)) / n
    for d, v in zip(dofs, vals):
        if v != 0:
            col = K[:, d - 1].toarray().ravel()
            b -= v * col
    pres = np.zeros(n, bool)
    pres[np.asarray(dofs, int) - 1] = True
    K = K.tolil()
    for d in np.nonzero(pres)[0]:
        K[:, d] = 0.0
        K[d, :] = 0.0
    for d, v in zip(dofs, vals):
        K[d - 1, d - 1] = m
        b[d - 1] = v * m
    return K.tocsc(), b


def boundary_dofs(mesh, cd, k: int, faceset: str = "boundary"):
    """Dofs of the field on the face set (vertex dofs of its faces, and face dofs for order 2)."""
    faces = set(int(f) for f in mesh.faceset(faceset))
    out = set()
    for c in range(mesh.ncells):
        for l, f in enumerate(mesh.cell_faces[c]):
            if int(f) not in faces:
                continue
            a, bb = ((1, 2), (2, 0), (0, 1))[l]   # local edge l joins these local vertices
            out.add(int(cd[c][a]))
            out.add(int(cd[c][bb]))
            if k == 2:
                out.add(int(cd[c][3 + l]))
    return np.array(sorted(out), dtype=np.int64)


def errornorm(mesh, k: int, u, u_ex, cd, qd: int | None = None) -> float:
    qd = k + 1 if qd is None else qd
    t = hdgref.tables(1, qd)
    qx, qy, qw = t["vx"], t["vy"], t["vw"]
    N, _ = lagrange_tables(k, qx, qy)
    s = 0.0
    for c in range(mesh.ncells):
        v = mesh.xy[mesh.cells[c] - 1]
        detJ = (v[1, 0] - v[0, 0]) * (v[2, 1] - v[0, 1]) - (v[2, 0] - v[0, 0]) * (v[1, 1] - v[0, 1])
        uc = np.asarray(u)[cd[c] - 1]
        for q in range(len(qw)):
            xq = (1 - qx[q] - qy[q]) * v[0] + qx[q] * v[1] + qy[q] * v[2]
            d = uc @ N[:, q] - hdgref.eval_field(u_ex, xq[0], xq[1])
            s += d * d * detJ * qw[q]
    return s


def solve_poisson_cg(mesh, k: int = 1, f=None, qd=None, kappa_cell=None):
    """The whole CG example: returns dict(K, b, Ka, ba, u, cell_dofs, err)."""
    f = hdgref.MANUFACTURED_F if f is None else f
    K, b, cd = assemble(mesh, k, f, qd, kappa_cell)
    dofs = boundary_dofs(mesh, cd, k)
    Ka, ba = apply_dirichlet(K, b, dofs, np.zeros(len(dofs)))
    u = spla.spsolve(Ka.tocsc(), ba)
    err = errornorm(mesh, k, u, hdgref.MANUFACTURED_U, cd, qd)
    return dict(K=K, b=b, Ka=Ka, ba=ba, u=u, cell_dofs=cd, dofs=dofs, err=err)
