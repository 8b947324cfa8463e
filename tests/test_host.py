"""CPU-only checks of the product's host side: the C ABI exports, the closed-form mesh numbering
against the oracle's first-visit numbering, the Triangle reader, and the triplet assembler."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def H():
    import __graft_entry__ as g
    g._build_module().build()
    return g.import_package()


def test_library_exports_every_declared_symbol(H):
    import ctypes
    src = open(os.path.join(ROOT, "include", "hdg.h")).read()
    names = set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(hdg_\w+)\s*\(", src, re.M))
    assert len(names) >= 30
    lib = ctypes.CDLL(os.path.join(ROOT, "hdiscontinuousgalerkin.jl_gb300", "libhdg.so"))
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each of them
    assert names <= set(H._lib.SIGNATURES), names - set(H._lib.SIGNATURES)


@pytest.mark.parametrize("nx,ny", [(1, 1), (2, 2), (3, 5), (7, 2), (10, 10), (32, 32), (17, 9)])
def test_rectangle_numbering_matches_oracle(H, oracle, nx, ny):
    m = H.rectangle_mesh(H.TriangleCell, (nx, ny), (0.0, 0.0), (1.0, 1.0), ctx=None)
    r = oracle.rectangle_mesh(nx, ny)
    assert m.ncells == r.ncells and m.nnodes == r.nnodes and m.nfaces == r.nfaces == nx + ny + 3 * nx * ny
    np.testing.assert_array_equal(H.getcells_matrix(m), r.cells)
    xy, cn, cf, fc = m._topology()
    np.testing.assert_array_equal(cf, r.cell_faces)
    np.testing.assert_array_equal(fc, r.faces)
    assert np.array_equal(xy, r.xy)  # bit-exact coordinates
    for name in ("boundary", "bottom", "right", "top", "left"):
        assert sorted(H.getfaceset(m, name)) == r.faceset(name).tolist()


def test_rectangle_other_box(H, oracle):
    m = H.rectangle_mesh(H.TriangleCell, (6, 4), (-1.5, 0.25), (2.0, 3.0), ctx=None)
    r = oracle.rectangle_mesh(6, 4, (-1.5, 0.25), (2.0, 3.0))
    assert np.array_equal(m._topology()[0], r.xy)
    assert sorted(H.getfaceset(m, "boundary")) == r.faceset("boundary").tolist()


def test_mesh_kats(H, kats, figure_root):
    m = H.parse_mesh_triangle(figure_root, ctx=None)
    assert H.getcells_matrix(m).tolist() == kats["figure2_1_cells"]
    assert H.get_vertices_matrix(m).tolist() == kats["figure2_1_vertices"]
    assert list(m.cells[0].faces) == kats["figure2_1_cell1_faces"]
    assert [H.face_orientation(m, 1, i) for i in (1, 2, 3)] == kats["figure2_1_cell1_orientation"]
    assert sorted(H.getfaceset(m, "boundary")) == kats["figure2_1_boundary"]
    assert H.cell_diameter(m, 1) == kats["figure2_1_cell1_diameter"]
    m = H.rectangle_mesh(H.TriangleCell, (2, 2), ctx=None)
    assert H.getcells_matrix(m).tolist() == kats["rect2x2_cells"]
    assert H.get_vertices_matrix(m).tolist() == kats["rect2x2_vertices"]
    assert list(m.cells[0].faces) == kats["rect2x2_cell1_faces"]
    assert [H.face_orientation(m, 1, i) for i in (1, 2, 3)] == kats["rect2x2_cell1_orientation"]
    assert sorted(H.getfaceset(m, "boundary")) == kats["rect2x2_boundary"]
    assert H.cell_diameter(m, 1) == kats["rect2x2_cell1_diameter"]


def test_triangle_reader_matches_oracle(H, oracle, figure_root):
    m = H.parse_mesh_triangle(figure_root, ctx=None)
    r = oracle.parse_mesh_triangle(figure_root)
    xy, cn, cf, fc = m._topology()
    np.testing.assert_array_equal(cn, r.cells)
    np.testing.assert_array_equal(cf, r.cell_faces)
    np.testing.assert_array_equal(fc, r.faces)


def test_triplet_assembler(H):
    import scipy.sparse as sp
    rng = np.random.default_rng(0)
    a = H.start_assemble(100)
    I, J, V = [], [], []
    for _ in range(40):
        edof = rng.choice(np.arange(1, 30), size=6, replace=False)
        Ke = rng.standard_normal((6, 6))
        H.assemble_(a, edof, Ke)
        for j in range(6):
            for i in range(6):
                I.append(edof[i] - 1); J.append(edof[j] - 1); V.append(Ke[i, j])
    K = H.end_assemble(a)
    ref = sp.csc_matrix((V, (I, J)), shape=K.shape)
    ref.sum_duplicates()
    ref.sort_indices()
    np.testing.assert_array_equal(K.colptr - 1, ref.indptr)
    np.testing.assert_array_equal(K.rowval - 1, ref.indices)
    np.testing.assert_allclose(K.nzval, ref.data, rtol=1e-15, atol=1e-15)
    g = np.zeros(10)
    H.assemble_(g, [1, 3, 3], [1.0, 2.0, 5.0])
    assert g[0] == 1.0 and g[2] == 7.0


def test_fields_host_eval(H, oracle):
    for f in (H.MANUFACTURED_F, H.Field.const(2.5), H.Field.bumps([[0.3, 0.4], [0.7, 0.2]], [0.1, 0.2], [1.0, -2.0]),
              H.Field.fourier(0.1, [[1, 2, 0.3, 0.5], [0, 3, 1.0, -0.2]], exponential=True)):
        for x, y in ((0.1, 0.2), (0.5, 0.9)):
            assert f(x, y) == pytest.approx(oracle.eval_field(f.as_oracle(), x, y), rel=1e-14)


def test_mesh_concat_offsets(H, oracle):
    """A batch mesh is the disjoint union of its problems' meshes, each with its own numbering."""
    parts = [H.rectangle_mesh(H.TriangleCell, (n, n), ctx=None) for n in (2, 3, 5)]
    u = H.concat_meshes(None, parts)
    node0, cell0, face0 = H.problem_offsets(u)
    assert node0.tolist() == [0, 9, 25, 61] and cell0.tolist() == [0, 8, 26, 76]
    xy, cn, cf, fc = u._topology()
    for k, n in enumerate((2, 3, 5)):
        r = oracle.rectangle_mesh(n, n)
        np.testing.assert_array_equal(cn[cell0[k]:cell0[k + 1]] - node0[k], r.cells)
        np.testing.assert_array_equal(cf[cell0[k]:cell0[k + 1]] - face0[k], r.cell_faces)
        f = fc[face0[k]:face0[k + 1]].copy()
        f[:, :2] -= node0[k]
        f[:, 2] -= cell0[k]
        f[:, 3] = np.where(f[:, 3] > 0, f[:, 3] - cell0[k], 0)
        np.testing.assert_array_equal(f, r.faces)
    b = sorted(H.getfaceset(u, "boundary"))
    ref = sorted(int(v) + int(face0[k]) for k, n in enumerate((2, 3, 5)) for v in oracle.rectangle_mesh(n, n).faceset("boundary"))
    assert b == ref


# ---- DofHandler (test/test_handlers.jl) and the sparsity-pattern assembler ------------------
def test_dofhandler_matches_reference_test(H):
    """The 2x2 P1 numbering, offsets, dof_range and boundary dofs of test/test_handlers.jl:6-18."""
    mesh = H.rectangle_mesh(H.TriangleCell, (2, 2), (0.0, 0.0), (1.0, 1.0), ctx=None)
    Wh = H.ScalarFunctionSpace(mesh, H.ContinuousLagrange(2, H.RefTetrahedron, 1), update_face_data=False)
    u_h = H.TrialFunction(Wh)
    dh = H.DofHandler([u_h], mesh)
    assert dh.cell_dofs.tolist() == [1, 2, 3, 2, 4, 3, 2, 5, 4, 5, 6, 4, 3, 4, 7, 4, 8, 7, 4, 6, 8, 6, 9, 8]
    assert dh.cell_dofs_offset.tolist() == [1, 4, 7, 10, 13, 16, 19, 22, 25]
    assert list(H.dof_range(dh, u_h)) == [1, 2, 3]
    dbc = H.Dirichlet(u_h, dh, "boundary", lambda x: 0.0)
    assert dbc.prescribed_dofs.tolist() == [1, 2, 3, 5, 6, 7, 8, 9]
    assert np.all(dbc.values == 0.0)


def test_dofhandler_p2_and_two_fields(H):
    """P2 adds one dof per face at its first visit; a second field is numbered after the first
    within each cell; the sparsity pattern holds every pair of dofs that share a cell."""
    mesh = H.rectangle_mesh(H.TriangleCell, (3, 2), (0.0, 0.0), (1.0, 1.0), ctx=None)
    nn, nf = mesh.nnodes, mesh.nfaces
    u = H.TrialFunction(H.ScalarFunctionSpace(mesh, H.ContinuousLagrange(2, H.RefTetrahedron, 2)))
    p = H.TrialFunction(H.ScalarFunctionSpace(mesh, H.ContinuousLagrange(2, H.RefTetrahedron, 1)))
    dh = H.DofHandler([u, p], mesh)
    assert H.ndofs(dh) == (nn + nf) + nn
    assert H.ndofs_per_cell(dh) == 9
    assert list(H.dof_range(dh, u)) == list(range(1, 7)) and list(H.dof_range(dh, p)) == [7, 8, 9]
    # first cell: vertices 1..3, faces 4..6, then the second field's vertices 7..9
    assert dh.cell_dofs[:9].tolist() == list(range(1, 10))
    K = H.create_sparsity_pattern(dh)
    dense = np.zeros(K.shape, bool)
    for c in range(mesh.ncells):
        g = dh.cell_dofs[dh.cell_dofs_offset[c] - 1: dh.cell_dofs_offset[c + 1] - 1] - 1
        dense[np.ix_(g, g)] = True
    dense |= np.eye(K.shape[0], dtype=bool)
    stored = np.zeros(K.shape, bool)
    for j in range(K.shape[1]):
        stored[K.indices[K.indptr[j]:K.indptr[j + 1]], j] = True
    assert np.array_equal(stored, dense) and K.nnz == dense.sum() and not K.data.any()
    Ks = H.create_symmetric_sparsity_pattern(dh)
    assert Ks.nnz == np.triu(dense).sum()


def test_pattern_assembler_matches_triplets(H):
    """start_assemble(K, f) + assemble! into a stored pattern equals the triplet assembler's
    sparse(I, J, V) on the same element matrices (src/assembler.jl:31-60 vs 97-137)."""
    rng = np.random.default_rng(5)
    mesh = H.rectangle_mesh(H.TriangleCell, (4, 3), (0.0, 0.0), (2.0, 1.0), ctx=None)
    u = H.TrialFunction(H.ScalarFunctionSpace(mesh, H.ContinuousLagrange(2, H.RefTetrahedron, 2)))
    dh = H.DofHandler([u], mesh)
    K = H.create_sparsity_pattern(dh)
    f = np.zeros(H.ndofs(dh))
    A = H.start_assemble(K, f)
    T = H.start_assemble(H.ndofs(dh))
    g = np.zeros(H.ndofs(dh))
    n = H.ndofs_per_cell(dh)
    dofs = np.zeros(n, np.int64)
    for c in range(1, mesh.ncells + 1):
        Ke = rng.standard_normal((n, n))
        fe = rng.standard_normal(n)
        H.celldofs_(dofs, dh, c)
        H.assemble_(A, dofs, Ke, fe)
        H.assemble_(T, dofs, Ke)
        H.assemble_(g, dofs, fe)
    ref = H.end_assemble(T).to_scipy().toarray()
    assert np.allclose(K.toarray(), ref, rtol=0, atol=1e-13)
    assert np.allclose(f, g, rtol=0, atol=1e-13)
    with pytest.raises(H.HDGError):
        H.assemble_(A, np.array([1, H.ndofs(dh)]), np.ones((2, 2)))


def test_unstructured_figure1_reader_matches_oracle(H, oracle):
    """The 62-cell unstructured Triangle mesh test/mesh/figure.1.*: the reader's cells, cell faces,
    face table, boundary set and orientations equal the oracle's restatement of
    src/triangle_mesh.jl (first-visit face numbering, edge-marker boundary)."""
    root = os.path.join(ROOT, "tests", "golden", "mesh", "figure.1")
    m = H.parse_mesh_triangle(root, ctx=None)
    om = oracle.parse_mesh_triangle(root)
    assert (m.nnodes, m.ncells, m.nfaces) == (om.nnodes, om.ncells, om.nfaces) == (41, 62, 102)
    xy, cn, cf, fc = m._topology()
    assert np.array_equal(xy, om.xy)
    assert np.array_equal(cn, om.cells) and np.array_equal(cf, om.cell_faces)
    assert np.array_equal(fc, om.faces)
    assert sorted(H.getfaceset(m, "boundary")) == sorted(om.faceset("boundary").tolist())
    for c in range(m.ncells):
        assert [H.face_orientation(m, c + 1, f + 1) for f in range(3)] == [om.orientation(c, f) for f in range(3)]


def test_generated_unstructured_mesh_reader_matches_oracle(H, oracle, tmp_path):
    """A Delaunay mesh written by tests/golden/make_unstructured_mesh.py (the generator of the
    at-scale GPU test, here with 42 x 42 points): its cells are counter-clockwise, its boundary
    edges are exactly the edges on the square's sides, and the library's reader gives the oracle's
    topology, first-visit face numbering, boundary set and orientations bit for bit."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_unstructured_mesh as gen
    xy, tri, edges, bnd = gen.unstructured_square(42, 7)
    a, b, c = xy[tri[:, 0]], xy[tri[:, 1]], xy[tri[:, 2]]
    assert np.all((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0]) > 0)
    mid = 0.5 * (xy[edges[:, 0]] + xy[edges[:, 1]])
    on_side = (np.isclose(mid[:, 0], 0) | np.isclose(mid[:, 0], 1) | np.isclose(mid[:, 1], 0)
               | np.isclose(mid[:, 1], 1))
    assert np.array_equal(on_side, bnd == 1)
    root = str(tmp_path / "sq")
    nc = gen.write_triangle_mesh(root, 42, 7)
    assert nc == len(tri) > 3000
    m = H.parse_mesh_triangle(root, ctx=None)
    om = oracle.parse_mesh_triangle(root)
    assert (m.nnodes, m.ncells, m.nfaces) == (om.nnodes, om.ncells, om.nfaces) == (42 * 42, nc, len(edges))
    xyl, cn, cf, fc = m._topology()
    assert np.array_equal(xyl, om.xy)
    assert np.array_equal(cn, om.cells) and np.array_equal(cf, om.cell_faces)
    assert np.array_equal(fc, om.faces)
    assert sorted(H.getfaceset(m, "boundary")) == sorted(om.faceset("boundary").tolist())
    assert len(H.getfaceset(m, "boundary")) == int(bnd.sum())
    for cc in range(0, m.ncells, 97):
        assert [H.face_orientation(m, cc + 1, f + 1) for f in range(3)] == [om.orientation(cc, f) for f in range(3)]


def test_write_vtk_roundtrip(H, tmp_path):
    """The headless output that stands in for the reference's Makie plot: a legacy VTK file whose
    points, triangles and fields read back as written."""
    m = H.rectangle_mesh(H.TriangleCell, (3, 2), (0.0, 0.0), (1.0, 1.0), ctx=None)
    xy, cn = m._topology()[0], m._topology()[1]
    u = xy[:, 0] * 2.0 + xy[:, 1]
    q = np.stack([xy[:, 1], -xy[:, 0]], axis=1)
    k = np.arange(cn.shape[0], dtype=float)
    path = tmp_path / "u.vtk"
    H.write_vtk(str(path), m, point_data={"u": u, "q": q}, cell_data={"kappa": k})
    lines = path.read_text().splitlines()
    i = lines.index(f"POINTS {xy.shape[0]} double")
    pts = np.array([[float(t) for t in ln.split()] for ln in lines[i + 1:i + 1 + xy.shape[0]]])
    assert np.array_equal(pts[:, :2], xy) and not pts[:, 2].any()
    i = lines.index(f"CELLS {cn.shape[0]} {4 * cn.shape[0]}")
    cells = np.array([[int(t) for t in ln.split()] for ln in lines[i + 1:i + 1 + cn.shape[0]]])
    assert (cells[:, 0] == 3).all() and np.array_equal(cells[:, 1:] + 1, cn)
    i = lines.index("SCALARS u double 1")
    assert np.array_equal(np.array([float(t) for t in lines[i + 2:i + 2 + xy.shape[0]]]), u)
    i = lines.index("SCALARS kappa double 1")
    assert np.array_equal(np.array([float(t) for t in lines[i + 2:i + 2 + cn.shape[0]]]), k)
    assert "VECTORS q double" in lines


def test_cg_oracle_pinned_by_reference_bound(oracle):
    """The CG Poisson oracle reproduces the reference's own bound on its 10 x 10 P1 example
    (test/test_CGExample.jl:92-93: squared L2 error <= 2e-4), and P2 converges further."""
    import cgref
    m = oracle.rectangle_mesh(10, 10)
    r1 = cgref.solve_poisson_cg(m, 1)
    assert r1["err"] <= 2e-4
    r2 = cgref.solve_poisson_cg(m, 2)
    assert r2["err"] < r1["err"] / 100
    # nodal basis: a partition of unity with Kronecker values at the nodes
    P = cgref.nodal_points(2)
    N, _ = cgref.lagrange_tables(2, P[:, 0], P[:, 1])
    assert np.allclose(N, np.eye(6), atol=1e-14)


@pytest.mark.parametrize("order", [1, 2])
def test_dofhandler_and_dirichlet_match_cg_oracle(H, oracle, order):
    """The library's DofHandler numbering and Dirichlet dofs equal the CG oracle's restatement of
    src/dofhandler.jl and src/boundary.jl:44-95 on a 6 x 5 mesh."""
    import cgref
    m = H.rectangle_mesh(H.TriangleCell, (6, 5), (0.0, 0.0), (1.0, 1.0), ctx=None)
    u = H.TrialFunction(H.ScalarFunctionSpace(m, H.ContinuousLagrange(2, H.RefTetrahedron, order)))
    dh = H.DofHandler([u], m)
    om = oracle.rectangle_mesh(6, 5)
    cd = cgref.distribute_dofs(om, order)
    assert np.array_equal(dh.cell_dofs.reshape(cd.shape), cd)
    dbc = H.Dirichlet(u, dh, "boundary", lambda x: 0.0)
    assert np.array_equal(dbc.prescribed_dofs, cgref.boundary_dofs(om, cd, order))


def test_bench_workload_generator_matches_library(H, oracle):
    """The batching workload that bench.py's reference arm builds with numpy and the oracle alone
    (no libhdg) is the one the GPU arm builds through the library: the same jittered coordinates
    (splitmix64 stream of hdg_mesh_jitter) and the same source parameters, bit for bit."""
    import bench
    specs = bench.c4_specs()
    probs = bench.c4_problems(H)
    assert len(specs) == len(probs) == 256
    for k in (0, 1, 17, 100, 255):
        s, pr = specs[k], probs[k]
        assert (s["n"], s["p"], s["qd"]) == (pr.n, pr.p, pr.qd())
        assert np.array_equal(np.asarray(pr.f.params), s["bumps"])
        assert np.array_equal(pr.kappa_cell, s["kappa_cell"])
        xy_lib = H.batch.host_mesh(pr)._topology()[0]
        om = oracle.rectangle_mesh(s["n"], s["n"])
        xy_np = bench.jitter_rect_xy(om.xy, s["n"], s["jitter"], s["seed"])
        assert np.array_equal(xy_lib, xy_np), k


def test_bench_cpu_sample_is_stratified():
    import bench
    specs = bench.c4_specs()
    idx = bench.c4_cpu_sample_indices(specs)
    assert len(idx) == len(set(idx)) == 48
    sizes = sorted(specs[k]["n"] for k in idx)
    alln = sorted(s["n"] for s in specs)
    assert sizes[0] <= alln[len(alln) // 40] and sizes[-1] >= alln[-len(alln) // 40 - 1]


def test_bench_roofline_selection():
    """The bench's roofline picks the kernel family with the most live time per step and, in it,
    the instance moving the most bytes; the level-0 sweep is reported beside it with the traffic
    of its committed ncu summary (stand-in bins: no GPU)."""
    import types
    import bench

    class Bin:
        def __init__(self, p, nd, l0, l1):
            self.p, self.ndofs, self.idx = p, nd, [0]
            self.mesh = types.SimpleNamespace(ncells=1000)
            self._s = {1: l0, 2: l1}

        def kernel_sample(self, which):
            ms, by, n = self._s[which]
            return {"ms": ms, "bytes": by, "launches": n}

    H = types.SimpleNamespace(PRECOND_AMG=1)
    bins = [Bin(1, 1000, (1.0, 1e9, 32), (2.0, 1e8, 56)), Bin(4, 5000, (1.5, 4e9, 32), (2.5, 3e8, 56))]
    B = types.SimpleNamespace(bins=bins, stats=[types.SimpleNamespace(iterations=100)])
    tims = [{"cg_samples": 8, "cg_a_ms": 0.1, "cg_a_bytes": 1e8, "element_ms": 5.0}] * 2
    rl, rle = bench.c4_rooflines(H, B, tims, 1, 6769.1, "measured")
    assert rl["family"] == "coarse sweeps" and "p=4 bin" in rl["kernel"]
    assert rl["family_ms_per_step"]["coarse sweeps"] > rl["family_ms_per_step"]["level-0 sweeps"]
    assert abs(rl["achieved"] - (3e8 / 56) / (2.5e-3 / 56) / 1e9) < 1e-9
    l0 = rl["level0_sweep"]
    assert "k_amg_face_cheb<5" in l0["kernel"] and l0["traffic"] == bench.profile_traffic("c4:k_amg_face_cheb<5>")
    assert l0["traffic"] is not None
    assert rle["bound"] == "fp64 pipe" and len(rle["bins"]) == 2
    assert abs(rle["elements_per_s"] - 2000 / 10e-3) < 1e-6 and rle["bins"][0]["elements_per_s"] == 1000 / 5e-3


@pytest.mark.parametrize("kind,prm,code,word", [
    (2, [3.0, 0.5, 0.5, 0.1, 1.0], -1, b"BUMPS"),        # K = 3 bumps, parameters for one
    (1, [1.0], -1, b"SINSIN"),                          # sin sin needs a, kx, ky
    (3, [2.0, 0.0, 1.0, 1.0, 0.0, 1.0], -1, b"FOURIER"),  # K = 2 modes, parameters for one
    (4, [-1.0, 0.0], -1, b"FOURIER"),                   # negative mode count
    (9, [1.0], -1, b"unknown kind"),
    (0, [], -1, b"CONST"),                              # a constant needs its value
    (0, [1.0] * 5000, -12, b"field parameters"),         # over the scratch capacity
])
def test_field_parameters_checked_before_device_work(H, kind, prm, code, word):
    """A field whose parameters do not cover what its kind reads is refused on the host, before any
    CUDA call (this runs without a GPU): the device evaluator would otherwise read past the
    parameters.  The no-allocation error norm also refuses a count over its fixed capacity."""
    import ctypes as C
    lib = H._lib.load()
    arr = np.ascontiguousarray(prm, dtype=np.float64) if prm else np.zeros(1)
    fc = H._lib.hdg_field(kind, len(prm), arr.ctypes.data_as(C.POINTER(C.c_double)))
    dummy = (C.c_double * 8)()
    out = C.c_double(-7.0)
    rc = lib.hdg_errornorm_l2sq_noalloc(0, None, 1, 0, 1, C.addressof(dummy), C.addressof(dummy),
                                        C.addressof(dummy), C.byref(fc), C.byref(out))
    assert rc == code
    assert word in lib.hdg_noalloc_last_error()
    assert out.value == -7.0


def test_reference_citations_point_inside_the_cited_files():
    """Every src/, examples/ or test/ citation with line numbers in the repository's sources and
    documents lies inside the cited reference file (skipped where the reference tree is absent)."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import check_citations as cc
    tree = cc.reference_tree([])
    if not tree:
        pytest.skip("reference tree not present")
    n, bad = cc.check(tree)
    assert n > 100
    assert not bad, "\n".join(bad)
