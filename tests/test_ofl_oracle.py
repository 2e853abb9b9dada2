"""The complex momentum-path oracle (restated optical-flux-lattice basis and
SpinlessFermionHamiltonian<dcmplx> build) pinned by identities: the momentum
sectors partition the N-particle space, the tables follow FindK1's momentum
rule, and the reference's Hermitian completion of the upper storage is
Hermitian when the tables' diagonal terms are real.  CPU only."""
from math import comb

import numpy as np
import pytest
import scipy.sparse as sp


@pytest.mark.parametrize("N,X,Y", [(3, 3, 4), (4, 2, 5), (2, 4, 4)])
def test_momentum_sectors_partition_the_space(oracle, N, X, Y):
    K = X * Y
    total = 0
    for kx in range(X):
        for ky in range(Y):
            b = oracle.basis_momentum(N, X, Y, kx, ky)
            total += len(b)
            assert all(int(b[i]) < int(b[i + 1]) for i in range(len(b) - 1))
            for w in b[:50]:
                ps = [p for p in range(K) if int(w) >> p & 1]
                assert len(ps) == N
                assert sum(p // Y for p in ps) % X == kx and sum(p % Y for p in ps) % Y == ky
    assert total == comb(K, N)


def test_tables_conserve_momentum(oracle):
    X, Y = 3, 4
    K = X * Y
    kt, vt = oracle.ofl_tables(X, Y, 3)
    assert len(kt) == len(vt) == (K + 1) * K * K // 2
    for k3 in range(K):
        for k4 in range(K):
            for k2 in range(K):
                k1 = oracle.ofl_k1(kt, K, k2, k3, k4)
                assert (k1 // Y + k2 // Y - k3 // Y - k4 // Y) % X == 0
                assert (k1 % Y + k2 % Y - k3 % Y - k4 % Y) % Y == 0
    # GetVkkkk reads the same entry for (k1,k2,k3,k4) and (k2,k1,k4,k3)
    assert oracle.ofl_v(vt, K, 5, 2, 7, 1) == oracle.ofl_v(vt, K, 2, 5, 1, 7)


@pytest.mark.parametrize("N,X,Y,kx,ky", [(3, 3, 4, 0, 0), (4, 3, 4, 1, 2), (4, 4, 4, 3, 1)])
def test_completion_is_hermitian(oracle, N, X, Y, kx, ky):
    K = X * Y
    kt, vt = oracle.ofl_tables(X, Y, 7)
    b = oracle.basis_momentum(N, X, Y, kx, ky)
    e = np.linspace(-0.3, 0.5, K).astype(complex)
    rp, col, val = oracle.build_upper_complex(b, K, kt, vt, e)
    assert np.all(col >= np.repeat(np.arange(len(b)), np.diff(rp)))          # upper storage
    M = oracle.complex_upper_to_full(rp, col, val, len(b))
    A = sp.csr_matrix((M[2], M[1], M[0]), shape=(len(b), len(b))).toarray()
    assert np.array_equal(A, A.conj().T)
    # the occupation energies enter the diagonal only
    rp0, col0, val0 = oracle.build_upper_complex(b, K, kt, vt)
    U = sp.csr_matrix((val, col, rp), shape=(len(b), len(b))).toarray()
    U0 = sp.csr_matrix((val0, col0, rp0), shape=(len(b), len(b))).toarray()
    off = ~np.eye(len(b), dtype=bool)
    assert np.array_equal(U[off], U0[off])
    occ = np.array([[int(w) >> k & 1 for k in range(K)] for w in b])
    assert np.allclose(np.diag(U) - np.diag(U0), occ @ e, atol=1e-13)


@pytest.mark.parametrize("N,X,Y,kx,ky", [(3, 3, 4, 0, 0), (5, 4, 5, 3, 2), (4, 4, 6, 1, 5)])
def test_c_restatement_matches_python(oracle, N, X, Y, kx, ky):
    """oracle.c's momentum basis, complex build and the reference's complex
    upper-triangle product (the CPU baseline) agree with the Python loops:
    basis and CRS bit for bit, product to rounding."""
    K = X * Y
    kt, vt = oracle.ofl_tables(X, Y, 5)
    e = np.linspace(-0.4, 0.6, K) + 1e-3j * np.arange(K)
    b = oracle.basis_momentum(N, X, Y, kx, ky)
    assert np.array_equal(oracle.basis_momentum_c(N, X, Y, kx, ky), b)
    a = oracle.build_upper_complex(b, K, kt, vt, e)
    c = oracle.build_upper_complex_c(b, K, kt, vt, e, nthreads=2)
    assert np.array_equal(a[0], c[0]) and np.array_equal(a[1], c[1])
    assert np.array_equal(a[2].view(np.uint64), c[2].view(np.uint64))
    M = oracle.complex_upper_to_full(*a, len(b))
    A = sp.csr_matrix((M[2], M[1], M[0]), shape=(len(b), len(b)))
    x = np.random.default_rng(1).uniform(-1, 1, len(b)) + 1j * np.random.default_rng(2).uniform(-1, 1, len(b))
    assert np.max(np.abs(oracle.cspmv_upper(*c, x, nthreads=2) - A @ x)) <= 1e-12 * np.abs(a[2]).max() * 50
