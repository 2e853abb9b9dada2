"""ed_residuals_noalloc: the allocation-free residual entry point.

Some callers of this library cannot let it call cudaMalloc: programs that hand
all device memory to their own pool allocator, and solver loops where a
cudaMalloc/cudaFree would synchronise the device.  For them
ed_residuals_noalloc computes the same residual norms as ed_residuals with its
scratch in a fixed file-scope device array.  Checked through the C ABI
against ed_residuals on two calls in a row (the second call reuses the array
the first one left behind)."""
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
