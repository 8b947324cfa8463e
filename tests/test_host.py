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
