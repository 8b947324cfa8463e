"""GPU parity: libhdg (CUDA, sm_103a) against the CPU oracle on the same inputs.

What is compared, and to what tolerance (FP64 path):
  * dof numbering and the CSC sparsity pattern: bit-exact;
  * element blocks K_e, b_e: within 1e-12 of the largest entry of the same cell's block (a cell's
    q rows scale like kappa/h and its u rows like 1, so one cell is the unit of scale);
  * every entry of the global trace matrix: within 1e-12 of the largest entry of the same row
    (relative to the row, so that small entries are checked on their own scale);
  * the Dirichlet diagonal that apply! writes (mean|diag K|): the reference sums the diagonal in
    sequence (src/boundary.jl:169-175) and so does the oracle, with a rounding error that grows
    with the number of dofs (bound N 2^-53); the device sums in a tree.  These entries are checked
    against that bound, and the device's value against the exactly summed mean to 1e-14;
  * the trace solution: the device solution (CG to 1e-12, then FP64 iterative refinement on a
    double-double residual, hdg_refine) is the solution of the oracle's system to a componentwise
    backward error max_i |b - K x|_i / (|K||x| + |b|)_i <= 1e-12 (measured 1e-16..1e-13): it
    solves a system within 1e-12 relative, entry by entry, of the oracle's.  The forward difference
    from the oracle's (refined) direct solution is bounded separately per case: the trace system's
    solution moves by 1e-13 (2*64^2 cells, p=2) to 3e-12 (2*256^2 cells) of its norm when the
    entries of K move by one unit in the last place (oracle test
    test_trace_solution_sensitivity_to_ulp_changes), and the device and oracle assemblies differ
    by a few such units, so two FP64 implementations agree on the solution only to that level;
    the reference's own direct solve (UMFPACK in Julia) differs from the refined solution by as
    much (the oracle's SuperLU: 2.7e-12 of the norm at 2*128^2 cells, p=2)."""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL_BLOCK = 1e-12
BWD_TOL = 1e-12


@pytest.fixture(scope="module")
def H():
    import __graft_entry__ as g
    g.build()
    return g.import_package()


def spaces(H, mesh, p, qd=None):
    fe = H.GenericFiniteElement(H.Dubiner(2, H.RefTetrahedron, p))
    Wh = H.ScalarFunctionSpace(mesh, fe, quad_degree=qd)
    Vh = H.VectorFunctionSpace(mesh, fe, quad_degree=qd)
    Mh = H.ScalarTraceFunctionSpace(Wh, H.GenericFiniteElement(H.Legendre(1, H.RefTetrahedron, p)))
    return Vh, Wh, Mh


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def rel_l2(a, b):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def block_rel(a, b):
    """max over entries of |a - b| / (largest |b| of the same cell's block); a, b: (cells, ...)."""
    a, b = np.asarray(a), np.asarray(b)
    scale = np.abs(b).reshape(len(b), -1).max(axis=1).reshape((len(b),) + (1,) * (b.ndim - 1))
    return float((np.abs(a - b) / np.maximum(scale, 1e-300)).max())


def row_rel(a, b):
    """max over entries of |a - b| / (largest |b| in the same row); a, b: (..., rows, cols)."""
    a, b = np.asarray(a), np.asarray(b)
    scale = np.abs(b).max(axis=-1, keepdims=True)
    return float((np.abs(a - b) / np.maximum(scale, 1e-300)).max())


def csc_parity(colptr, rowval, nzval, oK, dirichlet=None, diag_exact=None):
    """Pattern bit-exact, entries within RTOL_BLOCK of their row's largest entry; the Dirichlet
    diagonal (mean|diag K| after apply!) against the oracle's sequential-sum bound and, given the
    exactly summed mean diag_exact, the device's value to 1e-14.  Returns the measured figures."""
    np.testing.assert_array_equal(colptr, oK.indptr)
    np.testing.assert_array_equal(rowval, oK.indices)
    rows = np.asarray(oK.indices)
    cols = np.repeat(np.arange(oK.shape[0]), np.diff(oK.indptr))
    rowmax = np.zeros(oK.shape[0])
    np.maximum.at(rowmax, rows, np.abs(oK.data))
    d = np.abs(nzval - oK.data) / np.maximum(rowmax[rows], 1e-300)
    dd = np.zeros(len(d), bool)
    if dirichlet is not None and len(dirichlet):
        dm = np.zeros(oK.shape[0], bool)
        dm[np.asarray(dirichlet) - 1] = True
        dd = (rows == cols) & dm[rows]
    out = {"entries": float(d[~dd].max())}
    assert out["entries"] < RTOL_BLOCK, out
    if dd.any():
        n = oK.shape[0]
        out["dirichlet_diag"] = float(d[dd].max())
        assert out["dirichlet_diag"] <= n * 2.0 ** -53 + 1e-14, out
        if diag_exact is not None:
            got = nzval[dd]
            assert np.all(np.abs(got - diag_exact) <= 1e-14 * diag_exact), (got[:3], diag_exact)
    return out


def backward_error(oK, ob, x):
    """Componentwise backward error of x in the system oK x = ob (Oettli-Prager), with the residual
    summed in double-double (the oracle's csc_residual_dd)."""
    import hdgref
    r = hdgref.csc_residual_dd(oK, x, ob)
    den = abs(oK) @ np.abs(x) + np.abs(ob)
    return float((np.abs(r) / np.maximum(den, 1e-300)).max())


def check_solution(S, x, fwd_tol):
    """x (device trace solution) against the oracle system S (after apply!): componentwise backward
    error <= BWD_TOL, and relative L2 difference from the oracle's refined direct solution <= fwd_tol.
    Returns (the oracle's refined solution, measured figures)."""
    oK, ob = S.csc()
    xr = S.solve(refine=3)
    out = {"backward": backward_error(oK, ob, x), "forward": rel_l2(x, xr)}
    assert out["backward"] <= BWD_TOL, out
    assert out["forward"] <= fwd_tol, out
    return xr, out


def compare_system(H, oracle, mesh, omesh, p, qd=None, f=None, kappa=None, kappa_cell=None, tau=1.0, apply=True,
                   g=None, projection="reference", he_tau=False):
    f = f or H.MANUFACTURED_F
    Vh, Wh, Mh = spaces(H, mesh, p, qd)
    K, b, K_e, b_e = H.doassemble(Vh, Wh, Mh, tau, f, kappa=kappa, kappa_cell=kappa_cell, he_tau=he_tau)
    S = oracle.System(omesh, p, qd, tau, f.as_oracle(), kappa.as_oracle() if kappa is not None else None, kappa_cell,
                      he_tau=he_tau, threads=os.cpu_count() or 1)
    Ate, bte, Ke, be = K.element_blocks()
    oKe, obe = S.local()
    assert block_rel(Ke, oKe) < RTOL_BLOCK
    assert block_rel(be, obe) < RTOL_BLOCK
    oK0, _ = S.csc()
    diag_exact = math.fsum(np.abs(oK0.diagonal())) / oK0.shape[0]
    dofs = None
    if apply:
        dbc = H.Dirichlet(H.TrialFunction(Mh), mesh, "boundary", g, projection=projection)
        od, ov = S.dirichlet("boundary", g.as_oracle() if g is not None else None, projection=projection)
        np.testing.assert_array_equal(dbc.prescribed_dofs, od)
        np.testing.assert_allclose(dbc.values, ov, atol=1e-15)
        H.apply_(K, b, dbc)
        S.apply(od, ov)
        dofs = od
    colptr, rowval, nzval, rhs = K.csc(0)
    oK, ob = S.csc()
    csc_parity(colptr, rowval, nzval, oK, dofs, diag_exact if apply else None)
    assert rel(rhs, ob) < RTOL_BLOCK
    return K, S, (Vh, Wh, Mh)


def test_golden_figure21(H, oracle, kats, figure_root):
    """figure2.1, p=1, tau=1 (test/test_FunctionSpace.jl): blocks, matrix, solution, error bound."""
    mesh = H.parse_mesh_triangle(figure_root)
    omesh = oracle.parse_mesh_triangle(figure_root)
    K, S, (Vh, Wh, Mh) = compare_system(H, oracle, mesh, omesh, 1)
    uhat = H.solve(K, None, tol=1e-12, refine=2)
    ref, _ = check_solution(S, uhat, 1e-13)
    sigma_h, u_h, uhat_h = H.TrialFunction(Vh), H.TrialFunction(Wh), H.TrialFunction(Mh)
    K_e = H.system._LocalView(K, "K")
    H.get_usigma_(sigma_h, u_h, uhat_h, uhat, K_e, None, mesh)
    oq, ou, ouc = S.recover(ref)
    assert row_rel(u_h.m_values, ou) < 1e-12
    assert row_rel(sigma_h.m_values, oq) < 1e-12
    e = H.errornorm(u_h, H.MANUFACTURED_U)
    assert e == pytest.approx(oracle.errornorm(omesh, 1, ou, oracle.MANUFACTURED_U), rel=1e-10)
    assert e <= kats["figure2_1_errornorm_sq_max"]


def test_rect10_example_bound(H, oracle, kats):
    """examples/poisson2D_HDG.jl: 10x10, p=1, errornorm <= 6e-5."""
    mesh = H.rectangle_mesh(H.TriangleCell, (10, 10), (0.0, 0.0), (1.0, 1.0))
    uhat, q, u, st = H.solve_poisson(mesh, 1, H.MANUFACTURED_F, tol=1e-13)
    r = oracle.solve_poisson(oracle.rectangle_mesh(10, 10), 1)
    # the one-call flow stops the CG at 1e-13 (no refinement): its solution is still the oracle
    # system's to a componentwise backward error below 1e-12
    oK, ob = r["system"].csc()
    assert backward_error(oK, ob, uhat) <= BWD_TOL
    assert rel_l2(uhat, r["uhat"]) < 1e-12
    assert rel_l2(u, r["u"]) < 1e-12
    e = oracle.errornorm(oracle.rectangle_mesh(10, 10), 1, u, oracle.MANUFACTURED_U)
    assert e <= kats["rect10_errornorm_sq_max"]


@pytest.mark.parametrize("n,p,qd", [(2, 1, None), (4, 2, None), (8, 2, None), (5, 3, 6), (4, 4, 9), (32, 1, None),
                                    (16, 2, None)])
def test_rectangle_parity(H, oracle, n, p, qd):
    mesh = H.rectangle_mesh(H.TriangleCell, (n, n), (0.0, 0.0), (1.0, 1.0))
    omesh = oracle.rectangle_mesh(n, n)
    K, S, _ = compare_system(H, oracle, mesh, omesh, p, qd)
    uhat = H.solve(K, None, tol=1e-12, refine=2)
    assert K.stats.converged and K.refine_stats.converged
    # at these sizes (<= 2*32^2 cells) the two FP64 solutions agree to 1e-12 of the norm as well
    check_solution(S, uhat, 1e-12)


def test_non_square_box(H, oracle):
    mesh = H.rectangle_mesh(H.TriangleCell, (6, 3), (-1.0, 0.5), (2.0, 2.0))
    omesh = oracle.rectangle_mesh(6, 3, (-1.0, 0.5), (2.0, 2.0))
    compare_system(H, oracle, mesh, omesh, 2, f=H.Field.const(1.0))


def test_jitter_kappa_bumps(H, oracle):
    """The extensions of the precision/batching workloads: jittered nodes, kappa per cell or as
    exp(Fourier) field, Gaussian-bump source — against the oracle with the same inputs."""
    rng = np.random.default_rng(3)
    mesh = H.rectangle_mesh(H.TriangleCell, (8, 8), (0.0, 0.0), (1.0, 1.0))
    mesh.jitter(0.2, 11)
    omesh = oracle.rectangle_mesh(8, 8)
    omesh.set_xy(H.get_vertices_matrix(mesh))
    f = H.Field.bumps(rng.random((8, 2)), 0.05 + 0.1 * rng.random(8), rng.standard_normal(8))
    kc = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), mesh.ncells))
    compare_system(H, oracle, mesh, omesh, 2, f=f, kappa_cell=kc)
    modes = np.column_stack([rng.integers(-3, 4, 16), rng.integers(-3, 4, 16), rng.uniform(0, 6.28, 16),
                             rng.standard_normal(16) / 4])
    kap = H.Field.fourier(0.0, modes, exponential=True)
    compare_system(H, oracle, mesh, omesh, 3, qd=6, f=f, kappa=kap)


def test_convergence_rates(H):
    """L2 error of u against sin(pi x) sin(pi y): rate ~ p+1 (exact-enough quadrature for p >= 3)."""
    for p, qd in ((1, None), (2, None), (3, 6)):
        errs = []
        for n in (8, 16):
            mesh = H.rectangle_mesh(H.TriangleCell, (n, n), (0.0, 0.0), (1.0, 1.0))
            Vh, Wh, Mh = spaces(H, mesh, p, qd)
            K, b, K_e, b_e = H.doassemble(Vh, Wh, Mh, 1.0, H.MANUFACTURED_F)
            H.apply_(K, b, H.Dirichlet(H.TrialFunction(Mh), mesh, "boundary"))
            H.solve(K, b, tol=1e-13)
            K.recover()
            errs.append(math.sqrt(K.errornorm(H.MANUFACTURED_U)))
        rate = math.log2(errs[0] / errs[1])
        assert rate > p + 0.7, (p, errs, rate)


def _half_sin(H):
    """u = sin(pi x / 2) sin(pi y / 2), nonzero on x = 1 and y = 1, and f = -lap u."""
    return H.Field.sinsin(1.0, 0.5, 0.5), H.Field.sinsin(0.5 * math.pi ** 2, 0.5, 0.5)


@pytest.mark.parametrize("n,p,qd,tau", [(6, 1, None, 4.0), (5, 2, None, 0.25), (4, 3, 6, 10.0)])
@pytest.mark.parametrize("projection,he_tau", [("l2", True), ("l2", False), ("reference", True)])
def test_dirichlet_projection_and_he_tau_match_oracle(H, oracle, n, p, qd, tau, projection, he_tau):
    """The corrected trace Dirichlet projection and tau in He against the oracle's same options,
    with tau != 1 and nonzero boundary data."""
    u_ex, f = _half_sin(H)
    mesh = H.rectangle_mesh(H.TriangleCell, (n, n), (0.0, 0.0), (1.0, 1.0))
    omesh = oracle.rectangle_mesh(n, n)
    K, S, _ = compare_system(H, oracle, mesh, omesh, p, qd, f=f, tau=tau, g=u_ex, projection=projection,
                             he_tau=he_tau)
    if not he_tau and tau > 1:
        # He without tau and tau > 1: the trace matrix is indefinite on the free dofs (the oracle's
        # eigenvalues show positive ones), a system for a direct solver, not for CG
        return
    uhat = H.solve(K, None, tol=1e-12, refine=2)
    assert K.stats.converged
    check_solution(S, uhat, 1e-12)


def test_corrected_options_converge_with_boundary_data(H):
    """tau = 4 and u != 0 on the boundary: with the L2 trace projection and tau in He the error
    falls at rate p + 1, on the device.  (The reference's formulation gives an indefinite trace
    matrix at this tau and no convergence; the oracle's tests show both.)"""
    u_ex, f = _half_sin(H)
    for p, qd in ((1, None), (2, None)):
        e = []
        for n in (8, 16):
            mesh = H.rectangle_mesh(H.TriangleCell, (n, n), (0.0, 0.0), (1.0, 1.0))
            Vh, Wh, Mh = spaces(H, mesh, p, qd)
            K, b, _, _ = H.doassemble(Vh, Wh, Mh, 4.0, f, he_tau=True)
            H.apply_(K, b, H.Dirichlet(H.TrialFunction(Mh), mesh, "boundary", u_ex, projection="l2"))
            H.solve(K, b, tol=1e-13)
            K.recover()
            e.append(math.sqrt(K.errornorm(u_ex)))
        assert math.log2(e[0] / e[1]) > p + 0.7, e
        assert e[1] < 1e-3, e


def test_deterministic(H):
    mesh = H.rectangle_mesh(H.TriangleCell, (16, 16), (0.0, 0.0), (1.0, 1.0))
    outs = []
    for _ in range(2):
        uhat, q, u, st = H.solve_poisson(mesh, 2, H.MANUFACTURED_F, tol=1e-12)
        outs.append((uhat, u))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_reassemble_new_rhs(H, oracle):
    mesh = H.rectangle_mesh(H.TriangleCell, (6, 6), (0.0, 0.0), (1.0, 1.0))
    Vh, Wh, Mh = spaces(H, mesh, 2)
    K, b, _, _ = H.doassemble(Vh, Wh, Mh, 1.0, H.MANUFACTURED_F)
    K.reassemble(1.0, H.Field.const(3.0))
    S = oracle.System(oracle.rectangle_mesh(6, 6), 2, None, 1.0, (0, [3.0]))
    assert rel(K.csc()[3], S.csc()[1]) < RTOL_BLOCK


def test_error_paths(H):
    mesh = H.rectangle_mesh(H.TriangleCell, (4, 4), (0.0, 0.0), (1.0, 1.0))
    with pytest.raises(H.HDGError) as e:
        spaces(H, mesh, 4, 8)  # Strang/GM: an even order > 6 is not available (src/quadrature.jl:24)
    assert e.value.code == -3
    Vh, Wh, Mh = spaces(H, mesh, 1)
    with pytest.raises(H.HDGError) as e:
        H.Dirichlet(H.TrialFunction(Mh), mesh, "nowhere")
    assert e.value.code == -10
    K, b, _, _ = H.doassemble(Vh, Wh, Mh, 1.0, H.MANUFACTURED_F)
    H.apply_(K, b, H.Dirichlet(H.TrialFunction(Mh), mesh, "boundary"))
    with pytest.raises(H.HDGError) as e:
        H.solve(K, b, maxit=2, chunk=1)
    assert e.value.code == -5
    # a flipped cell: det(J) <= 0 (src/ScalarFunctionSpaces.jl:110)
    xy = H.get_vertices_matrix(mesh)
    xy[6] = xy[6] + np.array([0.6, 0.6])
    mesh.set_coordinates(xy)
    with pytest.raises(H.HDGError) as e:
        H.doassemble(Vh, Wh, Mh, 1.0, H.MANUFACTURED_F)
    assert e.value.code == -2


@pytest.mark.parametrize("n,p,qd", [(32, 2, None), (16, 3, 6)])
def test_mixed_precision_solve(H, oracle, n, p, qd):
    """FP32 Krylov iteration with FP64 reliable updates reaches the FP64 tolerance: the solution
    agrees with the FP64 solve and with the oracle's direct solve."""
    mesh = H.rectangle_mesh(H.TriangleCell, (n, n), (0.0, 0.0), (1.0, 1.0))
    Vh, Wh, Mh = spaces(H, mesh, p, qd)
    K, b, _, _ = H.doassemble(Vh, Wh, Mh, 1.0, H.MANUFACTURED_F)
    H.apply_(K, b, H.Dirichlet(H.TrialFunction(Mh), mesh, "boundary"))
    u64 = H.solve(K, b, tol=1e-11)
    it64 = K.stats.iterations
    # the FP32 operator limits the attainable true residual to ~1e-12 on these systems
    umx = H.solve(K, b, tol=1e-10, precision=H.PREC_MIXED)
    assert K.stats.converged and K.stats.rel_residual <= 1e-10
    assert K.stats.iterations < 3 * it64
    S = oracle.System(oracle.rectangle_mesh(n, n), p, qd, 1.0, H.MANUFACTURED_F.as_oracle())
    S.apply(*S.dirichlet())
    ref = S.solve()
    assert rel(umx, ref) < 1e-8
    assert rel(umx, u64) < 1e-8


def test_batch_matches_single_problems(H, oracle):
    """A degree-binned batch (uneven sizes, p = 1..4, jitter, per-cell kappa, bump sources) gives
    each problem the solution of the oracle run on that problem alone."""
    rng = np.random.default_rng(7)
    probs = []
    for k, (n, p) in enumerate([(4, 1), (7, 2), (3, 3), (5, 4), (6, 1), (2, 2), (4, 3)]):
        f = H.Field.bumps(rng.random((8, 2)), 0.1 + 0.1 * rng.random(8), rng.standard_normal(8))
        kc = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), 2 * n * n))
        probs.append(H.Problem(n=n, p=p, f=f, kappa_cell=kc, jitter=0.2, seed=100 + k))
    ctx = H.default_context()
    for prec, tol, rtol in ((H.PREC_FP64, 1e-12, 1e-10), (H.PREC_MIXED, 1e-10, 1e-8)):
        B = H.Batch(ctx, probs, precision=prec)
        stats = B.solve(tol=tol)
        assert all(s.converged for s in stats)
        sols = B.solutions()
        for pr, (uh, q, u) in zip(probs, sols):
            om = oracle.rectangle_mesh(pr.n, pr.n)
            hm = H.batch.host_mesh(pr)
            om.set_xy(hm._topology()[0])
            r = oracle.solve_poisson(om, pr.p, qd=pr.qd(), f=pr.f.as_oracle(), kappa_cell=pr.kappa_cell)
            assert rel(uh, r["uhat"]) < rtol, (pr.n, pr.p, prec)
            assert rel(u, r["u"]) < rtol * 10


@pytest.mark.parametrize("copies", [0, 1])
def test_serving_same_alone_and_in_mix(H, monkeypatch, copies):
    """Continuous batching: every request's result is the same when served alone and when served
    in a mix of requests of several sizes and degrees (resident and new meshes), within 1e-8.  With
    copies = 1 the requests on resident meshes run on the engine's device-resident systems
    (HDG_ENGINE_RESIDENT_COPIES): two resident meshes get a second request with another source
    and coefficient, which waits for the first and then reuses its system (reassembly, the
    multigrid hierarchy built for the first request's matrix)."""
    monkeypatch.setenv("HDG_ENGINE_RESIDENT_COPIES", str(copies))
    rng = np.random.default_rng(11)
    ctx = H.default_context()
    specs = []
    for k, (n, p) in enumerate([(6, 1), (9, 2), (4, 3), (5, 4), (8, 2), (3, 1), (7, 3), (6, 2)]):
        f = H.Field.bumps(rng.random((8, 2)), 0.05 + 0.1 * rng.random(8), 10 * rng.standard_normal(8))
        kc = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), 2 * n * n))
        specs.append((H.Problem(n=n, p=p, f=f, kappa_cell=kc, jitter=0.2, seed=500 + k)))
    resident = list(range(len(specs)))[::2]
    extra = []  # (mesh index, source, kappa) of the second requests on two resident meshes
    for i in resident[:2]:
        pr = specs[i]
        f2 = H.Field.bumps(rng.random((8, 2)), 0.05 + 0.1 * rng.random(8), 10 * rng.standard_normal(8))
        extra.append((i, f2, pr.kappa_cell[::-1].copy()))

    def serve(reqs, resident_ids):
        eng = H.Engine(ctx, hbm_budget_gb=8, max_batch=8, max_flights=4, tol=1e-11)
        mids = {i: eng.add_resident(H.batch.host_mesh(specs[i]), specs[i].p) for i in resident_ids}
        rid = []
        for i, f, kc in reqs:
            pr = specs[i]
            if i in mids:
                rid.append(eng.submit(pr.p, f, kc, mesh_id=mids[i]))
            else:
                rid.append(eng.submit(pr.p, f, kc, mesh=H.batch.host_mesh(pr)))
        done = eng.run_until_idle()
        assert len(done) == len(reqs) and all(d["converged"] for d in done)
        return [eng.result(r) for r in rid]

    reqs = [(i, specs[i].f, specs[i].kappa_cell) for i in range(len(specs))] + extra
    mix = serve(reqs, resident)
    for (i, f, kc), got in zip(reqs, mix):
        alone = serve([(i, f, kc)], [])[0]
        for a, b in zip(got, alone):
            assert rel(a, b) < 1e-8, i


@pytest.mark.gpu
@pytest.mark.parametrize("n,p,qd,var", [(10, 1, None, False), (16, 2, None, True), (12, 3, 6, True), (8, 4, 9, True)])
def test_multigrid_solution_matches_oracle(H, oracle, n, p, qd, var):
    """The multigrid-preconditioned CG (FP64 CG, FP32 smoothed-aggregation V-cycle) reaches the
    same trace solution as the oracle's direct solve, in fewer iterations than Jacobi-PCG."""
    rng = np.random.default_rng(n * 10 + p)
    kc = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), 2 * n * n)) if var else None
    f = H.Field.bumps(rng.random((8, 2)), 0.1 + 0.1 * rng.random(8), rng.standard_normal(8))
    pr = H.Problem(n=n, p=p, f=f, kappa_cell=kc, jitter=0.2 if var else 0.0, seed=3)
    hm = H.batch.host_mesh(pr)
    mesh = H.rectangle_mesh(H.TriangleCell, (n, n), (0.0, 0.0), (1.0, 1.0))
    mesh.set_coordinates(hm._topology()[0])
    q_deg = qd if qd else p + 1
    fe = H.GenericFiniteElement(H.Dubiner(2, H.RefTetrahedron, p))
    Wh = H.ScalarFunctionSpace(mesh, fe, quad_degree=q_deg)
    Vh = H.VectorFunctionSpace(mesh, fe, quad_degree=q_deg)
    Mh = H.ScalarTraceFunctionSpace(Wh, H.GenericFiniteElement(H.Legendre(1, H.RefTetrahedron, p)))
    K, b, _, _ = H.doassemble(Vh, Wh, Mh, 1.0, f, kappa_cell=kc)
    dbc = H.Dirichlet(H.TrialFunction(Mh), mesh, "boundary")
    H.apply_(K, b, dbc)
    u_mg = K.solve(tol=1e-12, preconditioner=H.PRECOND_AMG)
    it_mg = K.stats.iterations
    K.reassemble(1.0, f, kappa_cell=kc)
    K.apply_dirichlet(dbc.prescribed_dofs, dbc.values)
    u_j = K.solve(tol=1e-12)
    it_j = K.stats.iterations
    om = oracle.rectangle_mesh(n, n)
    om.set_xy(hm._topology()[0])
    r = oracle.solve_poisson(om, p, qd=q_deg, f=f.as_oracle(), kappa_cell=kc)
    assert rel(u_mg, r["uhat"]) < 1e-10, (rel(u_mg, r["uhat"]), it_mg)
    assert rel(u_mg, u_j) < 1e-10
    assert it_mg < it_j / 2, (it_mg, it_j)  # the gap widens with the mesh size (see the benches)


@pytest.mark.gpu
def test_multigrid_batch_matches_single_problems(H, oracle):
    """A degree-binned batch solved with the multigrid preconditioner (each problem its own
    hierarchy inside the shared arrays) gives each problem the oracle's solution."""
    rng = np.random.default_rng(7)
    probs = []
    for k, (n, p) in enumerate([(4, 1), (7, 2), (3, 3), (5, 4), (6, 1), (2, 2), (4, 3), (12, 2)]):
        f = H.Field.bumps(rng.random((8, 2)), 0.1 + 0.1 * rng.random(8), rng.standard_normal(8))
        kc = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), 2 * n * n))
        probs.append(H.Problem(n=n, p=p, f=f, kappa_cell=kc, jitter=0.2, seed=100 + k))
    B = H.Batch(H.default_context(), probs, precision=H.PREC_FP64)
    stats = B.solve(tol=1e-12, preconditioner=H.PRECOND_AMG)
    assert all(s.converged for s in stats)
    for pr, (uh, q, u) in zip(probs, B.solutions()):
        om = oracle.rectangle_mesh(pr.n, pr.n)
        om.set_xy(H.batch.host_mesh(pr)._topology()[0])
        r = oracle.solve_poisson(om, pr.p, qd=pr.qd(), f=pr.f.as_oracle(), kappa_cell=pr.kappa_cell)
        assert rel(uh, r["uhat"]) < 1e-10, (pr.n, pr.p)


@pytest.mark.parametrize("pc", ["jacobi", "amg"])
def test_pipelined_step_equals_sequential_calls(H, pc):
    """hdg_batch_step (per-bin streams: assembly, apply!, CG and recovery overlapped across bins)
    gives bit-identical results to the same work done call by call: reassembly, apply!,
    hdg_solve_batch and recovery of each bin in turn.  Repeated resident steps repeat the result."""
    import ctypes as C
    L = H._lib
    rng = np.random.default_rng(21)
    probs = []
    for k, (n, p) in enumerate([(9, 1), (5, 2), (4, 3), (3, 4), (6, 2), (7, 4)]):
        f = H.Field.bumps(rng.random((8, 2)), 0.1 + 0.1 * rng.random(8), rng.standard_normal(8))
        kc = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), 2 * n * n))
        probs.append(H.Problem(n=n, p=p, f=f, kappa_cell=kc, jitter=0.2, seed=700 + k))
    pcv = H.PRECOND_AMG if pc == "amg" else H.PRECOND_JACOBI
    B = H.Batch(H.default_context(), probs, precision=H.PREC_MIXED)
    st1 = B.solve(tol=1e-10, reassemble=True, preconditioner=pcv)
    s1 = B.solutions()
    st2 = B.solve(tol=1e-10, reassemble="resident", preconditioner=pcv)
    s2 = B.solutions()
    # call by call
    for b in B.bins:
        b.reassemble(resident=True)
        b.apply()
    o = L.hdg_solver(1e-10, 100000, int(H.PREC_MIXED), 32, 1e-5, int(pcv))
    st = (L.hdg_stats * len(probs))()
    arr = (C.c_void_p * len(B.bins))(*[b.h for b in B.bins])
    assert L.load().hdg_solve_batch(len(B.bins), arr, C.byref(o), st) == 0
    for b in B.bins:
        b.recover()
    s3 = B.solutions()
    for a, b_, c in zip(s1, s2, s3):
        for x, y, z in zip(a, b_, c):
            assert np.array_equal(x, y) and np.array_equal(x, z)
    assert [s.iterations for s in st1] == [s.iterations for s in st2]
    # in-step downloads into page-locked arrays give the same arrays as the copies afterwards
    B.solve(tol=1e-10, reassemble="resident", preconditioner=pcv, download=True)
    s4 = [tuple(np.array(x) for x in t) for t in B.solutions(downloaded=True)]
    for a, d in zip(s1, s4):
        for x, y in zip(a, d):
            assert np.array_equal(x, y)
    for a, d in zip(B.solutions(), s4):
        for x, y in zip(a, d):
            assert np.array_equal(x, y)
    # a solve without apply! is refused; assembly without apply! is refused
    assert L.load().hdg_batch_step(len(B.bins), arr, C.byref(o), L.STEP_ASSEMBLE, st) == -1  # HDG_ERR_ARG


@pytest.mark.parametrize("p,qd", [(1, None), (2, None), (3, 6)])
def test_unstructured_figure1_parity(H, oracle, p, qd):
    """The unstructured figure.1 mesh: trace matrix, solution and recovery equal the oracle's, and the
    manufactured solution is approximated (squared L2 error small and shrinking with p)."""
    root = os.path.join(os.path.dirname(__file__), "golden", "mesh", "figure.1")
    mesh = H.parse_mesh_triangle(root)
    omesh = oracle.parse_mesh_triangle(root)
    K, S, (Vh, Wh, Mh) = compare_system(H, oracle, mesh, omesh, p, qd=qd)
    uhat = H.solve(K, None, tol=1e-12, refine=2)
    ref, _ = check_solution(S, uhat, 1e-12)
    q, u, _ = K.recover()
    oq, ou, _ = S.recover(ref)
    assert rel_l2(u, ou) < 1e-12 and rel_l2(q, oq) < 1e-12
    e = K.errornorm(H.MANUFACTURED_U)
    assert e == pytest.approx(oracle.errornorm(omesh, p, ou, oracle.MANUFACTURED_U, qd=qd), rel=1e-9)
    assert e < {1: 1e-3, 2: 1e-4, 3: 1e-5}[p]


def test_nodal_avg(H, oracle):
    """nodal_avg(u_h) (src/DiscreteFunctions.jl:81-95): the per-node mean of the recovered u over
    the node's cells equals the same average formed on the host from the oracle's Dubiner basis,
    and approximates the exact solution at the nodes."""
    n, p = 10, 2
    mesh = H.rectangle_mesh(H.TriangleCell, (n, n), (0.0, 0.0), (1.0, 1.0))
    Vh, Wh, Mh = spaces(H, mesh, p, None)
    K, b, K_e, b_e = H.doassemble(Vh, Wh, Mh, 1.0, H.MANUFACTURED_F)
    H.apply_(K, b, H.Dirichlet(H.TrialFunction(Mh), mesh, "boundary"))
    uhat = H.solve(K, b, tol=1e-13)
    sigma_h, u_h, uhat_h = H.TrialFunction(Vh), H.TrialFunction(Wh), H.TrialFunction(Mh)
    H.get_usigma_(sigma_h, u_h, uhat_h, uhat, H.system._LocalView(K, "K"), None, mesh)
    got = H.nodal_avg(u_h)
    xy, cn = H.get_vertices_matrix(mesh), H.getcells_matrix(mesh)
    nw = (p + 1) * (p + 2) // 2
    vals = np.array([[oracle.dubiner(a + 1, vx, vy)[0] for vx, vy in ((0, 0), (1, 0), (0, 1))] for a in range(nw)])
    acc, cnt = np.zeros(len(xy)), np.zeros(len(xy))
    for c in range(mesh.ncells):
        for k in range(3):
            acc[cn[c, k] - 1] += u_h.m_values[c] @ vals[:, k]
            cnt[cn[c, k] - 1] += 1
    assert rel(got, acc / cnt) < 1e-12
    exact = np.sin(np.pi * xy[:, 0]) * np.sin(np.pi * xy[:, 1])
    assert np.max(np.abs(got - exact)) < 2e-3


@pytest.mark.parametrize("n,order,var", [(10, 1, False), (12, 2, False), (9, 1, True), (7, 2, True)])
def test_cg_poisson_path_matches_oracle(H, oracle, n, order, var):
    """examples/poisson2D_CG.jl on the device: the stiffness values and load assembled into the
    DofHandler's pattern, the system after apply!, the PCG solution and errornorm equal the CG
    oracle's (jittered mesh and per-cell kappa in the variable cases); the 10 x 10 P1 example
    meets the reference's bound errornorm <= 2e-4 (test/test_CGExample.jl:92-93)."""
    import cgref
    rng = np.random.default_rng(n * 3 + order)
    mesh = H.rectangle_mesh(H.TriangleCell, (n, n), (0.0, 0.0), (1.0, 1.0))
    om = oracle.rectangle_mesh(n, n)
    kc = None
    if var:
        pr = H.Problem(n=n, p=order, f=H.MANUFACTURED_F, jitter=0.2, seed=17)
        xy = H.batch.host_mesh(pr)._topology()[0]
        mesh.set_coordinates(xy)
        om.set_xy(xy)
        kc = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), 2 * n * n))
    Wh = H.ScalarFunctionSpace(mesh, H.ContinuousLagrange(2, H.RefTetrahedron, order), update_face_data=False)
    u_h = H.TrialFunction(Wh)
    dh = H.DofHandler([u_h], mesh)
    K0 = H.create_sparsity_pattern(dh)
    dbc = H.Dirichlet(u_h, dh, "boundary", lambda x: 0.0)
    K, b = H.doassemble_cg(Wh, K0, dh, H.MANUFACTURED_F, kappa_cell=kc)
    Kref, bref, cd = cgref.assemble(om, order, oracle.MANUFACTURED_F, kappa_cell=kc)
    assert np.array_equal(dh.cell_dofs.reshape(cd.shape), cd)
    Kd = K.csc()
    scale = abs(Kref).max()
    assert abs(Kd - Kref).max() <= 1e-13 * scale
    assert np.abs(b - bref).max() <= 1e-13 * np.abs(bref).max()
    H.apply_(K, b, dbc)
    Ka, ba = cgref.apply_dirichlet(Kref, bref, dbc.prescribed_dofs, dbc.values)
    assert abs(K.csc() - Ka).max() <= 1e-13 * scale
    assert np.abs(b - ba).max() <= 1e-13 * np.abs(ba).max()
    u = H.solve(K, b, tol=1e-13)
    assert K.stats.converged
    uref = cgref.spla.spsolve(Ka.tocsc(), ba)
    assert rel(u, uref) < 1e-10
    H.reconstruct_(u_h, u, dh)
    assert np.array_equal(u_h.m_values, u[cd - 1])
    err = H.errornorm(u_h, H.MANUFACTURED_U)
    eref = cgref.errornorm(om, order, uref, oracle.MANUFACTURED_U, cd)
    assert abs(err - eref) <= 1e-8 * eref
    if (n, order, var) == (10, 1, False):
        assert err <= 2e-4


def test_cg_poisson_path_refuses_bad_inputs(H):
    """doassemble_cg refuses a pattern that lacks an element coupling (HDG_ERR_ARG from
    hdg_lagrange_create), an order whose DofHandler numbering is incomplete, and an inverted cell
    (HDG_ERR_NEG_DETJ)."""
    import scipy.sparse as sp
    mesh = H.rectangle_mesh(H.TriangleCell, (4, 4), (0.0, 0.0), (1.0, 1.0))
    Wh = H.ScalarFunctionSpace(mesh, H.ContinuousLagrange(2, H.RefTetrahedron, 1), update_face_data=False)
    u_h = H.TrialFunction(Wh)
    dh = H.DofHandler([u_h], mesh)
    K = H.create_sparsity_pattern(dh)
    diag_only = sp.identity(K.shape[0], format="csc")
    with pytest.raises(H.HDGError):
        H.doassemble_cg(Wh, diag_only, dh, H.MANUFACTURED_F)
    W3 = H.ScalarFunctionSpace(mesh, H.ContinuousLagrange(2, H.RefTetrahedron, 3), update_face_data=False)
    u3 = H.TrialFunction(W3)
    dh3 = H.DofHandler([u3], mesh)
    with pytest.raises(NotImplementedError):
        H.doassemble_cg(W3, H.create_sparsity_pattern(dh3), dh3, H.MANUFACTURED_F)
    xy = mesh._topology()[0].copy()
    cn = mesh._topology()[1]
    a, b = cn[0, 1] - 1, cn[0, 2] - 1
    xy[[a, b]] = xy[[b, a]]          # swap two vertices of the first cell: it turns inside out
    mesh.set_coordinates(xy)
    with pytest.raises(H.HDGError):
        H.doassemble_cg(Wh, K, dh, H.MANUFACTURED_F)


@pytest.mark.parametrize("n,fwd", [(64, 1e-11), (128, 4e-11)])
def test_scaled_manufactured_parity(H, oracle, n, fwd):
    """The scaled plain configuration (manufactured Poisson, p = 2, tau = 1, FP64) at 2*64^2 and
    2*128^2 cells: CSC pattern bit-exact, matrix, rhs and element blocks entry by entry, the trace
    solution (Jacobi-PCG to 1e-12 + refinement) in backward error and against the per-size forward
    bound, and the recovered q and u."""
    mesh = H.rectangle_mesh(H.TriangleCell, (n, n), (0.0, 0.0), (1.0, 1.0))
    omesh = oracle.rectangle_mesh(n, n)
    K, S, _ = compare_system(H, oracle, mesh, omesh, 2)
    uhat = H.solve(K, None, tol=1e-12, refine=2)
    assert K.stats.converged and K.refine_stats.converged
    ref, m = check_solution(S, uhat, fwd)
    q, u, _ = K.recover()
    oq, ou, _ = S.recover(ref)
    assert rel_l2(q, oq) <= fwd and rel_l2(u, ou) <= fwd


def test_precision_config_shape_parity(H, oracle):
    """The precision configuration's ingredients on 2*128^2 cells: p = 3, interior nodes jittered by
    U(-0.2h, 0.2h), kappa = exp(g) with g 64 random Fourier modes (wavelength >= 0.1, RMS 1), a
    random smooth Fourier source; the FP64 device assembly against the oracle's entry by entry and
    the trace solution in backward error."""
    import bench
    n, p, qd = 128, 3, 6
    mesh = H.rectangle_mesh(H.TriangleCell, (n, n), (0.0, 0.0), (1.0, 1.0))
    mesh.jitter(0.2, 4242)
    omesh = oracle.rectangle_mesh(n, n)
    omesh.set_xy(H.get_vertices_matrix(mesh))
    kappa, f = bench.c3_fields(H)
    K, S, _ = compare_system(H, oracle, mesh, omesh, p, qd, f=f, kappa=kappa)
    uhat = H.solve(K, None, tol=1e-12, preconditioner=H.PRECOND_AMG, refine=2)
    ref, m = check_solution(S, uhat, 1e-9)
    q, u, _ = K.recover()
    oq, ou, _ = S.recover(ref)
    assert rel_l2(u, ou) <= 1e-9 and rel_l2(q, oq) <= 1e-9


@pytest.mark.parametrize("p", [1, 2])
def test_unstructured_at_scale_parity(H, oracle, tmp_path, p):
    """Triangle-format ingestion at scale: a 100,352-cell jittered Delaunay mesh of the unit square
    written by tests/golden/make_unstructured_mesh.py, read by parse_mesh_triangle on both sides;
    numbering and face sets bit-exact, trace matrix entry by entry, trace solution in backward error."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_unstructured_mesh as gen
    root = str(tmp_path / "square")
    assert gen.write_triangle_mesh(root, 225, 2024) >= 100_000
    mesh = H.parse_mesh_triangle(root)
    omesh = oracle.parse_mesh_triangle(root)
    xy, cn, cf, fc = mesh._topology()
    assert np.array_equal(cf, omesh.cell_faces) and np.array_equal(fc, omesh.faces) and np.array_equal(xy, omesh.xy)
    assert sorted(H.getfaceset(mesh, "boundary")) == omesh.faceset("boundary").tolist()
    K, S, _ = compare_system(H, oracle, mesh, omesh, p)
    uhat = H.solve(K, None, tol=1e-12, preconditioner=H.PRECOND_AMG, refine=2)
    ref, m = check_solution(S, uhat, 1e-10)
    q, u, _ = K.recover()
    oq, ou, _ = S.recover(ref)
    assert rel_l2(u, ou) <= 1e-10


_TAIL_SCRIPT = r"""
import os, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import __graft_entry__ as g
H = g.import_package()
rng = np.random.default_rng(11)
probs = []
for k, (n, p) in enumerate([(64, 2), (24, 2), (48, 2), (16, 3), (40, 3)]):
    f = H.Field.bumps(rng.random((8, 2)), 0.05 + 0.1 * rng.random(8), 10 * rng.standard_normal(8))
    kc = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), 2 * n * n))
    probs.append(H.Problem(n=n, p=p, f=f, kappa_cell=kc, jitter=0.2, seed=300 + k))
B = H.Batch(H.default_context(), probs, precision=H.PREC_MIXED)
stats = B.solve(tol=1e-9, preconditioner=H.PRECOND_AMG)
assert all(s.converged for s in stats)
np.savez(sys.argv[2], its=np.array([s.iterations for s in stats]),
         **{f"u{k}": np.concatenate([np.ravel(a) for a in sol]) for k, sol in enumerate(B.solutions())})
"""


def test_multigrid_cycle_variants_are_bit_identical(tmp_path):
    """The V-cycle's launch shapes that the autotuner chooses between give the same bits: the
    coarse levels cycled by one k_amg_tail launch per V-cycle (one CTA per problem) or by one launch
    per kernel per level (HDG_AMG_TAIL_ROWS), and the level-0 smoother with a thread per face or per
    row (HDG_AMG_SWEEP); the tuned default too."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    script = tmp_path / "cycle.py"
    script.write_text(_TAIL_SCRIPT)
    out = {}
    for name, env_add in (("plain", {"HDG_AMG_TAIL_ROWS": "0", "HDG_AMG_SWEEP": "face"}),
                          ("tail", {"HDG_AMG_TAIL_ROWS": "1024", "HDG_AMG_SWEEP": "row"}),
                          ("tuned", {})):
        env = dict(os.environ, HDG_AMG_VERBOSE="1", **env_add)
        for k in ("HDG_AMG_TAIL_ROWS", "HDG_AMG_SWEEP"):
            if k not in env_add:
                env.pop(k, None)
        r = subprocess.run([sys.executable, str(script), root, str(tmp_path / f"{name}.npz")], env=env,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        out[name] = (np.load(tmp_path / f"{name}.npz"), r.stderr)
    assert "tail from level 0" in out["plain"][1]
    assert "tail from level 2" in out["tail"][1] or "tail from level 3" in out["tail"][1], out["tail"][1][-1000:]
    assert "amg tune:" in out["tuned"][1]
    a = out["plain"][0]
    for name in ("tail", "tuned"):
        b = out[name][0]
        np.testing.assert_array_equal(a["its"], b["its"])
        for k in a.files:
            assert a[k].tobytes() == b[k].tobytes(), (name, k)
