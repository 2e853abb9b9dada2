"""Thick-restart basis rotation (K7): the tensor-core digit-splitting product
against the FP64 product and an extended-precision product of the same data."""
import ctypes

import numpy as np
import pytest

from hamiltonian_diagonalization_gb300 import _capi as C

pytestmark = pytest.mark.gpu


def rotate(torch, V, Y, k, method):
    n, m = V.shape
    Vd = torch.from_numpy(np.asfortranarray(V).ravel(order="F").copy()).cuda()
    out = torch.empty(n * k, dtype=torch.float64, device="cuda")
    Yf = np.asfortranarray(Y)
    st = C.lib().ed_basis_rotate(ctypes.c_void_p(Vd.data_ptr()), n, m,
                                 Yf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), Y.shape[0], k,
                                 ctypes.c_void_p(out.data_ptr()), method)
    return st, out.cpu().numpy().reshape(k, n).T


@pytest.mark.parametrize("n,m,k", [(100003, 41, 25), (70001, 29, 16), (65536, 64, 40), (9000, 16, 4)])
def test_tensor_rotation_matches_fp64(cuda, n, m, k):
    torch = cuda
    rng = np.random.default_rng(m)
    V = rng.standard_normal((n, m)) * np.exp(rng.uniform(-12, 0, (n, 1)))   # rows of different scale
    V[5] = 0.0                                                                # a zero row
    V[:, 2] *= 1e-7
    Y = rng.standard_normal((m, m))
    Y[:, 1] = 0.0                                                             # a zero column
    st1, out1 = rotate(torch, V, Y, k, 1)
    st2, out2 = rotate(torch, V, Y, k, 2)
    assert st1 == 0 and st2 == 0
    # extended-precision reference on a row sample (long double is software
    # quad on some hosts), always including the zero row
    rows = np.unique(np.concatenate([[5], rng.choice(n, 1500, replace=False)]))
    Vs = V[rows]
    exact = (Vs.astype(np.longdouble) @ Y[:, :k].astype(np.longdouble)).astype(np.float64)
    scale = np.abs(Vs).max(axis=1)[:, None] * np.abs(Y[:, :k]).max(axis=0)[None, :]
    scale[scale == 0] = 1.0
    err1 = np.max(np.abs(out1[rows] - exact) / scale)
    err2 = np.max(np.abs(out2[rows] - exact) / scale)
    # the two methods agree everywhere to the same bound
    full_scale = np.abs(V).max(axis=1)[:, None] * np.abs(Y[:, :k]).max(axis=0)[None, :]
    full_scale[full_scale == 0] = 1.0
    assert np.max(np.abs(out2 - out1) / full_scale) <= 8e-15
    assert err1 <= 4e-15, err1
    assert err2 <= 4e-15, err2          # at least as accurate as FP64 FMAs
    assert np.all(out2[5] == 0.0) and np.all(out2[:, 1] == 0.0)
    # the register-digit kernel and the shared-memory one give the same bits
    st3, out3 = rotate(torch, V, Y, k, 3)
    assert st3 == 0 and np.array_equal(out2, out3)


@pytest.mark.parametrize("n,m,k", [(1371535, 41, 17), (1371535, 41, 10), (20011, 48, 32), (5003, 33, 9), (17, 5, 3)])
def test_register_and_shared_digit_kernels_agree(cuda, n, m, k):
    # the headline's restart shapes and edge sizes: bit-identical results
    torch = cuda
    rng = np.random.default_rng(n + m + k)
    V = rng.standard_normal((n, m)) * np.exp(rng.uniform(-6, 0, (n, 1)))
    Y = rng.standard_normal((m, m))
    st2, out2 = rotate(torch, V, Y, k, 2)
    st3, out3 = rotate(torch, V, Y, k, 3)
    assert st2 == 0 and st3 == 0 and np.array_equal(out2, out3)


def test_tensor_rotation_rejects_large_m(cuda):
    torch = cuda
    V = np.ones((1000, 65))
    Y = np.ones((65, 65))
    st, _ = rotate(torch, V, Y, 10, 2)
    assert st == 1   # ED_ERR_ARG
