"""The no-allocation error norm, hdg_errornorm_l2sq_noalloc.

It serves callers that cannot allocate device memory: an embedding runtime that owns the device
heap, or code in a region where allocation is forbidden.  It must give the same squared L2 error
as hdg_errornorm_l2sq on the same recovered solution, on two calls in a row.  Its scratch array is
shared by every call and keeps the last call's contents, so the second call checks that the
reduction ticket is cleared.  The file name sorts last, so every other test has run before it."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def H():
    import __graft_entry__ as g
    g.build()
    return g.import_package()


@pytest.mark.parametrize("n,p,qd", [(8, 2, None), (6, 3, 6), (5, 4, 9)])
def test_noalloc_errornorm_matches(H, n, p, qd):
    import torch
    mesh = H.rectangle_mesh(H.TriangleCell, (n, n), (0.0, 0.0), (1.0, 1.0))
    fe = H.GenericFiniteElement(H.Dubiner(2, H.RefTetrahedron, p))
    Wh = H.ScalarFunctionSpace(mesh, fe, quad_degree=qd)
    Vh = H.VectorFunctionSpace(mesh, fe, quad_degree=qd)
    Mh = H.ScalarTraceFunctionSpace(Wh, H.GenericFiniteElement(H.Legendre(1, H.RefTetrahedron, p)))
    K, b, _, _ = H.doassemble(Vh, Wh, Mh, 1.0, H.MANUFACTURED_F)
    H.apply_(K, b, H.Dirichlet(H.TrialFunction(Mh), mesh, "boundary"))
    H.solve(K, b, tol=1e-12)
    _, u_h, _ = K.recover()
    expected = K.errornorm(H.MANUFACTURED_U)  # the allocating entry point
    # caller-owned device inputs: allocated by the caller, not by the library
    xy = torch.tensor(H.get_vertices_matrix(mesh), dtype=torch.float64, device="cuda")
    cells = torch.tensor(H.getcells_matrix(mesh) - 1, dtype=torch.int32, device="cuda")
    ud = torch.tensor(u_h, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    lib = H._lib.load()
    fc = H.MANUFACTURED_U.as_c()
    for _ in range(2):
        out = C.c_double(-1.0)
        rc = lib.hdg_errornorm_l2sq_noalloc(0, None, p, qd or 0, mesh.ncells, xy.data_ptr(), cells.data_ptr(),
                                            ud.data_ptr(), C.byref(fc), C.byref(out))
        assert rc == 0, lib.hdg_noalloc_last_error()
        # The squared error sums d^2 with d = u_h - u_ex, about 3e-6 at p = 4.  The two kernels
        # are compiled separately, and a rounding difference of 1e-16 in u_h(x_q) moves d^2 by
        # about 1e-10 relative, so the bound is 1e-9 (at p = 2, 3 they agree to 1e-12).
        assert out.value == pytest.approx(expected, rel=1e-9, abs=1e-300)


def test_noalloc_rejects_oversized_requests(H):
    import torch
    lib = H._lib.load()
    xy = torch.zeros((3, 2), dtype=torch.float64, device="cuda")
    cells = torch.zeros((1, 3), dtype=torch.int32, device="cuda")
    ud = torch.zeros((1, 3), dtype=torch.float64, device="cuda")
    big = np.zeros(5000)
    fc = H._lib.hdg_field(H._lib.FIELD_CONST, big.size, big.ctypes.data_as(C.POINTER(C.c_double)))
    out = C.c_double(0.0)
    rc = lib.hdg_errornorm_l2sq_noalloc(0, None, 1, 0, 1, xy.data_ptr(), cells.data_ptr(), ud.data_ptr(),
                                        C.byref(fc), C.byref(out))
    assert rc == -12  # HDG_ERR_CAPACITY
    assert b"field parameters" in lib.hdg_noalloc_last_error()
