"""The device eigensolver of the projected problems (cyclic Jacobi, one CTA per
matrix) against numpy's eigh: eigenvalues, residuals and orthonormality, on
random, arrowhead-plus-tridiagonal (a thick restart's shape), degenerate,
diagonal and zero matrices."""
import ctypes

import numpy as np
import pytest

from hamiltonian_diagonalization_gb300 import _capi as C

pytestmark = pytest.mark.gpu

F64 = ctypes.POINTER(ctypes.c_double)


def device_eigh(mats):
    mats = np.ascontiguousarray(mats, dtype=np.float64)
    count, m, _ = mats.shape
    ev = np.empty((count, m))
    vec = np.empty((count, m, m))
    C.check(C.lib().ed_sym_eigen_batched(m, count, mats.ctypes.data_as(F64), ev.ctypes.data_as(F64),
                                         vec.ctypes.data_as(F64)))
    return ev, vec.transpose(0, 2, 1)      # [count][row][column]


def restart_shape(rng, m):
    k = m // 3
    A = np.zeros((m, m))
    A[np.arange(k), np.arange(k)] = np.sort(rng.standard_normal(k)) + 20.0
    A[:k, k] = A[k, :k] = rng.standard_normal(k) * 1e-3
    for j in range(k, m):
        A[j, j] = 20.0 + rng.standard_normal()
    for j in range(k, m - 1):
        A[j, j + 1] = A[j + 1, j] = rng.uniform(0.5, 2.0)
    return A


@pytest.mark.parametrize("m", [1, 2, 3, 17, 29, 41, 64, 101, 128])
def test_device_eigh_matches_numpy(cuda, m):
    rng = np.random.default_rng(m)
    mats = []
    B = rng.standard_normal((m, m))
    mats.append(B + B.T)
    mats.append(restart_shape(rng, m) if m > 3 else np.diag(rng.standard_normal(m)))
    Q, _ = np.linalg.qr(rng.standard_normal((m, m)))
    d = np.repeat(rng.standard_normal((m + 2) // 3), 3)[:m]            # threefold eigenvalues
    mats.append(Q @ np.diag(d) @ Q.T)
    mats.append(np.diag(rng.standard_normal(m)))
    mats.append(np.zeros((m, m)))
    mats = np.array(mats)
    ev, vec = device_eigh(mats)
    for A, e, V in zip(mats, ev, vec):
        scale = max(1.0, np.abs(A).max())
        w = np.linalg.eigvalsh(A)
        assert np.all(np.diff(e) >= 0)
        assert np.max(np.abs(e - w)) <= 1e-13 * scale
        assert np.max(np.abs(A @ V - V * e)) <= 1e-13 * scale
        assert np.max(np.abs(V.T @ V - np.eye(m))) <= 1e-13


def test_device_eigh_rejects_oversized(cuda):
    a = np.zeros(129 * 129)
    out = np.empty(129 * 129)
    st = C.lib().ed_sym_eigen_batched(129, 1, a.ctypes.data_as(F64), out.ctypes.data_as(F64), out.ctypes.data_as(F64))
    assert st == C.ED_ERR_RANGE
