"""ed_residuals_noalloc: the allocation-free residual entry point.

Some callers of this library cannot let it call cudaMalloc: programs that hand
all device memory to their own pool allocator, and solver loops where a
cudaMalloc/cudaFree would synchronise the device.  For them
ed_residuals_noalloc computes the same residual norms as ed_residuals with its
scratch in a fixed file-scope device array.  Checked through the C ABI
against ed_residuals and against numpy residuals of the oracle's matrix, on
two calls in a row each (the second call reuses the array the first one left
behind), on a small sector and on one large enough that the row blocks reach
their cap."""
import ctypes

import numpy as np
import pytest

import hamiltonian_diagonalization_gb300 as ed
from hamiltonian_diagonalization_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def _op_for(H):
    op = ctypes.c_void_p()
    C.check(C.lib().ed_op_from_crs(H.m_crsSparseMatrix._h, ctypes.byref(op)))
    return op


def _residuals(fn, op, X, lam):
    k = len(lam)
    out = np.empty(k)
    st = fn(op, ctypes.c_void_p(X.data_ptr()), lam.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), k,
            out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return st, out


def test_noalloc_residuals_match_allocating_entry(cuda):
    torch = cuda
    L = C.lib()
    H = ed.SpinlessFermionHamiltonian()
    H.Initialize(8, 22, twoLz=0)
    H.Add_CdCdCC_Terms(ed.QuarticTermTables(22, ed.odd_coulomb_list(22)))
    n = H.GetDimension()
    op = _op_for(H)
    try:
        rng = np.random.default_rng(123)
        for call in range(2):
            k = 5 if call == 0 else 3
            X = torch.from_numpy(rng.uniform(-1, 1, n * k)).cuda()
            lam = rng.uniform(10.0, 14.0, k)
            st_a, ref = _residuals(L.ed_residuals, op, X, lam)
            st_b, got = _residuals(L.ed_residuals_noalloc, op, X, lam)
            assert st_a == 0 and st_b == 0, C.lib().ed_last_error()
            assert np.all(ref > 0)
            assert np.max(np.abs(got - ref) / ref) <= 1e-12, (got, ref)
    finally:
        L.ed_op_free(op)


def test_noalloc_residuals_match_numpy(cuda, oracle):
    # the same residuals from the oracle's matrix (the restated reference
    # build) on the host, two calls in a row
    import scipy.sparse as sp
    torch = cuda
    L = C.lib()
    N, norb = 8, 22
    pp = ed.odd_coulomb_list(norb)
    H = ed.SpinlessFermionHamiltonian()
    H.Initialize(N, norb, twoLz=0)
    H.Add_CdCdCC_Terms(ed.QuarticTermTables(norb, pp))
    n = H.GetDimension()
    b = oracle.basis(N, norb, 0)
    kt, vt = oracle.quartic_tables(norb, pp)
    rp, col, val = oracle.build_upper(b, norb, kt, vt)
    U = sp.csr_matrix((val, col, rp), shape=(n, n))
    A = (U + U.T - sp.diags(U.diagonal())).tocsr()
    op = _op_for(H)
    try:
        rng = np.random.default_rng(7)
        for k in (4, 2):
            Xh = rng.uniform(-1, 1, (k, n))
            lam = rng.uniform(10.0, 14.0, k)
            X = torch.from_numpy(np.ascontiguousarray(Xh.ravel())).cuda()
            st, got = _residuals(L.ed_residuals_noalloc, op, X, lam)
            assert st == 0, L.ed_last_error()
            ref = np.linalg.norm(A @ Xh.T - Xh.T * lam, axis=0)
            assert np.max(np.abs(got - ref) / ref) <= 1e-12, (got, ref)
    finally:
        L.ed_op_free(op)


def test_noalloc_residuals_match_on_a_large_sector(cuda):
    # N=11, 2S=30 (1,371,535 rows): the row blocks reach their cap of four
    # per SM, so the cross-block sum runs over hundreds of partials
    torch = cuda
    L = C.lib()
    H = ed.SpinlessFermionHamiltonian()
    H.Initialize(11, 31, twoLz=0)
    H.Add_CdCdCC_Terms(ed.QuarticTermTables(31, ed.odd_coulomb_list(31)))
    n = H.GetDimension()
    assert n > 2048 * 4 * torch.cuda.get_device_properties(0).multi_processor_count
    op = _op_for(H)
    try:
        rng = np.random.default_rng(9)
        for k in (3, 2):
            X = torch.from_numpy(rng.uniform(-1, 1, n * k)).cuda()
            lam = rng.uniform(20.0, 23.0, k)
            st_a, ref = _residuals(L.ed_residuals, op, X, lam)
            st_b, got = _residuals(L.ed_residuals_noalloc, op, X, lam)
            assert st_a == 0 and st_b == 0, L.ed_last_error()
            assert np.max(np.abs(got - ref) / ref) <= 1e-12, (got, ref)
    finally:
        L.ed_op_free(op)
        del H


def test_noalloc_rejects_beyond_its_limits(cuda):
    torch = cuda
    L = C.lib()
    H = ed.SpinlessFermionHamiltonian()
    H.Initialize(4, 12, twoLz=0)
    H.Add_CdCdCC_Terms(ed.QuarticTermTables(12, [0.0, 1.0]), store_upper=True)
    n = H.GetDimension()
    op = _op_for(H)
    try:
        X = torch.zeros(n * 65, dtype=torch.float64, device="cuda")
        st, _ = _residuals(L.ed_residuals_noalloc, op, X, np.zeros(65))
        assert st == C.ED_ERR_ARG and b"1..64" in L.ed_last_error()
        st, _ = _residuals(L.ed_residuals_noalloc, op, X, np.zeros(2))     # upper-triangle storage
        assert st == C.ED_ERR_ARG and b"full-storage" in L.ed_last_error()
    finally:
        L.ed_op_free(op)
    H2 = ed.SpinlessFermionHamiltonian()
    H2.Initialize(4, 12, twoLz=0)
    H2.Add_CdCdCC_Terms(ed.QuarticTermTables(12, [0.0, 1.0]))
    op = _op_for(H2)
    try:
        xh = np.zeros(H2.GetDimension())                               # x on the host
        st, _ = _residuals(L.ed_residuals_noalloc, op, torch.from_numpy(xh), np.zeros(1))
        assert st == C.ED_ERR_ARG and b"current device" in L.ed_last_error()
    finally:
        L.ed_op_free(op)
