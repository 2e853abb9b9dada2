"""H*v on the device (stored CRS in both storages, matrix-free) against the
oracle's restatement of SymmetricMatrixVectorMultiply; tolerance 1e-13
relative to |H| |x| (different FP64 summation order)."""
import numpy as np
import pytest

import hamiltonian_diagonalization_gb300 as ed

pytestmark = pytest.mark.gpu


def setup(N, norb, tlz, pp, upper=False, matfree=False):
    H = ed.SpinlessFermionHamiltonian()
    H.Initialize(N, norb, twoLz=tlz)
    T = ed.QuarticTermTables(norb, pp)
    H.Add_CdCdCC_Terms(T, store_upper=upper, matrix_free=matfree)
    return H, T


def apply(torch, H, x):
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    ed.MatrixVectorFunction(H).Simple(xd, yd)
    torch.cuda.synchronize()
    return yd.cpu().numpy()


# (3, 40, 1): more than 36 orbitals, the matrix-free product on the main rank
# tables; the others use its compact shared-memory tables
@pytest.mark.parametrize("case", [(4, 10, 0), (6, 16, 4), (8, 22, 0), (10, 28, 2), (3, 40, 1)])
def test_products_match_oracle(cuda, oracle, case):
    N, norb, tlz = case
    pp = oracle.odd_coulomb_list(norb)
    b = oracle.basis(N, norb, tlz)
    kt, vt = oracle.quartic_tables(norb, pp)
    urp, ucol, uval = oracle.build_upper(b, norb, kt, vt)
    x = np.random.default_rng(5).uniform(-1, 1, len(b))
    yref = oracle.spmv_sym_upper(urp, ucol, uval, x)
    scale = np.abs(uval).max() * np.abs(x).max() * 50
    for kw in ({"upper": False}, {"upper": True}, {"matfree": True}):
        H, _ = setup(N, norb, tlz, pp, **kw)
        y = apply(cuda, H, x)
        assert np.max(np.abs(y - yref)) <= 1e-13 * scale, kw


@pytest.mark.parametrize("case", [(4, 10, 0), (6, 16, 4), (8, 22, 0), (10, 28, 2), (2, 9, 2), (3, 9, 0)])
def test_row_kernels_match_oracle(cuda, oracle, case):
    # every full-storage kernel (row lanes, shared-reduction rows, sliced ELL, fixed point) on
    # every sector, including ones with fewer rows than a tile and with empty rows
    torch = cuda
    N, norb, tlz = case
    pp = oracle.odd_coulomb_list(norb)
    b = oracle.basis(N, norb, tlz)
    kt, vt = oracle.quartic_tables(norb, pp)
    urp, ucol, uval = oracle.build_upper(b, norb, kt, vt)
    x = np.random.default_rng(6).uniform(-1, 1, len(b))
    yref = oracle.spmv_sym_upper(urp, ucol, uval, x)
    scale = np.abs(uval).max() * np.abs(x).max() * 50
    H, _ = setup(N, norb, tlz, pp)
    xd = torch.from_numpy(x).cuda()
    for kernel in range(1, 9):
        yd = torch.full_like(xd, np.nan)
        H.m_crsSparseMatrix.multiply(xd, yd, kernel)
        torch.cuda.synchronize()
        assert np.max(np.abs(yd.cpu().numpy() - yref)) <= 1e-13 * scale, kernel
    Hu, _ = setup(N, norb, tlz, pp, upper=True)
    with pytest.raises(ed.EDError):
        Hu.m_crsSparseMatrix.multiply(xd, torch.empty_like(xd), 2)


def test_linearity_and_symmetry_at_scale(cuda, oracle):
    N, norb, tlz = 11, 31, 0
    pp = oracle.odd_coulomb_list(norb)
    H, _ = setup(N, norb, tlz, pp)
    n = H.GetDimension()
    rng = np.random.default_rng(9)
    x, z = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    hx, hz = apply(cuda, H, x), apply(cuda, H, z)
    hxz = apply(cuda, H, 0.5 * x - 2.0 * z)
    assert np.max(np.abs(hxz - (0.5 * hx - 2.0 * hz))) <= 1e-12 * np.max(np.abs(hx))
    assert abs(z @ hx - x @ hz) <= 1e-12 * abs(z @ hx) + 1e-9
    # matrix-free regenerates the same operator
    Hm, _ = setup(N, norb, tlz, pp, matfree=True)
    hxm = apply(cuda, Hm, x)
    assert np.max(np.abs(hxm - hx)) <= 1e-12 * np.max(np.abs(hx))


def test_aliasing_rejected(cuda, oracle):
    H, _ = setup(4, 10, 0, [0.0, 1.0])
    x = cuda.zeros(H.GetDimension(), dtype=cuda.float64, device="cuda")
    with pytest.raises(ed.EDError):
        ed.MatrixVectorFunction(H).Simple(x, x)


# ------------------------------------------------ the fixed-point integer kernel

def _fix_ints(v):
    """The kernel's fixed-point integers A = round(v 2^(1080 - E)) (nearest,
    ties away from zero) and E, the largest biased exponent field (at least 1)."""
    b = np.ascontiguousarray(v, dtype=np.float64).view(np.uint64)
    e = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    m = (b & np.uint64((1 << 52) - 1)).astype(np.int64) + np.where(e > 0, 1 << 52, 0)
    ee = np.maximum(e, 1)
    E = int(ee.max()) if len(ee) else 1
    sh = ee - E + 5
    q = np.zeros(len(m), dtype=np.int64)
    pos = sh >= 0
    q[pos] = m[pos] << sh[pos]
    neg = (sh < 0) & (sh > -64)
    k = -sh[neg]
    q[neg] = (m[neg] + (np.int64(1) << (k - 1))) >> k
    sign = (b >> np.uint64(63)).astype(bool)
    return np.where(sign, -q, q), E


def _fix_product(rowptr, col, val, x):
    """The exactly rounded y_i = round(sum_j A_ij X_j 2^(ea + ex - 2160))."""
    A, ea = _fix_ints(val)
    X, ex = _fix_ints(x)
    prod = [int(a) * int(xx) for a, xx in zip(A.tolist(), X[col].tolist())]
    y = np.empty(len(rowptr) - 1)
    for i in range(len(y)):
        S = sum(prod[rowptr[i]:rowptr[i + 1]])
        sc = ea + ex - 2160
        # int / int true division rounds once, to nearest even (subnormals included)
        y[i] = S / (1 << -sc) if sc < 0 else float(S << sc)
    return y


@pytest.mark.parametrize("case", [(6, 16, 4), (8, 22, 0), (3, 9, 0)])
def test_fixed_point_product_is_exactly_rounded(cuda, case):
    # bit equality with the exact integer sum rounded once, on inputs with
    # zeros, both signs, a wide exponent range and subnormals
    torch = cuda
    N, norb, tlz = case
    H, _ = setup(N, norb, tlz, ed.odd_coulomb_list(norb))
    rp, col, val = H.m_crsSparseMatrix.to_host()
    n = len(rp) - 1
    rng = np.random.default_rng(11)
    xs = [rng.uniform(-1, 1, n),
          rng.standard_normal(n) * np.exp(rng.uniform(-40, 5, n)),
          np.where(rng.random(n) < 0.3, 0.0, rng.uniform(-1e-300, 1e-300, n)) * 1e-10,
          np.zeros(n)]
    xs[1][::7] = 0.0
    for x in xs:
        xd = torch.from_numpy(x).cuda()
        ref = _fix_product(rp, col, val, x).view(np.uint64)
        for kernel in (6, 7, 8):       # rows in registers, staged in shared memory, sliced ELL
            yd = torch.full_like(xd, np.nan)
            H.m_crsSparseMatrix.multiply(xd, yd, kernel)
            torch.cuda.synchronize()
            assert np.array_equal(yd.cpu().numpy().view(np.uint64), ref), kernel


def test_fixed_point_product_error_below_fp64(cuda):
    # against the exact product of the FP64 inputs (rational arithmetic on a
    # row sample): the fixed-point kernel's error is far below the FP64
    # kernel's, element by element in sum and in the largest
    from fractions import Fraction
    torch = cuda
    H, _ = setup(10, 28, 2, ed.odd_coulomb_list(28))
    rp, col, val = H.m_crsSparseMatrix.to_host()
    n = len(rp) - 1
    x = np.random.default_rng(12).standard_normal(n)
    x /= np.linalg.norm(x)
    xd = torch.from_numpy(x).cuda()
    ys = {}
    for kernel in (2, 6):
        yd = torch.empty_like(xd)
        H.m_crsSparseMatrix.multiply(xd, yd, kernel)
        torch.cuda.synchronize()
        ys[kernel] = yd.cpu().numpy()
    rows = np.random.default_rng(13).choice(n, 400, replace=False)
    err = {2: [], 6: []}
    for i in rows:
        exact = sum(Fraction(float(val[k])) * Fraction(float(x[col[k]])) for k in range(rp[i], rp[i + 1]))
        for kernel in (2, 6):
            err[kernel].append(abs(float(Fraction(float(ys[kernel][i])) - exact)))
    assert sum(err[6]) <= 0.5 * sum(err[2])
    assert max(err[6]) <= max(err[2])


def test_fixed_point_product_edges(cuda):
    torch = cuda
    H, _ = setup(10, 28, 2, ed.odd_coulomb_list(28))   # 188 elements a row on average
    n = H.GetDimension()
    x = np.random.default_rng(14).uniform(-1, 1, n)
    x[17] = np.nan
    xd = torch.from_numpy(x).cuda()
    yd = torch.zeros_like(xd)
    H.m_crsSparseMatrix.multiply(xd, yd, 6)
    torch.cuda.synchronize()
    assert np.all(np.isnan(yd.cpu().numpy()))       # a non-finite entry of x: every entry NaN
    # the default product of this one-level sector is the fixed-point kernel
    x[17] = 0.25
    xd = torch.from_numpy(x).cuda()
    y6, y0 = torch.empty_like(xd), torch.empty_like(xd)
    H.m_crsSparseMatrix.multiply(xd, y6, 6)
    H.m_crsSparseMatrix.multiply(xd, y0, 0)
    torch.cuda.synchronize()
    assert torch.equal(y6, y0)
    Hu, _ = setup(10, 28, 2, ed.odd_coulomb_list(28), upper=True)
    with pytest.raises(ed.EDError):
        Hu.m_crsSparseMatrix.multiply(xd, torch.empty_like(xd), 6)


def test_staged_product_matches_at_scale_and_wait_runs_out(cuda):
    # the headline sector: the staged kernel gives the register kernel's bits;
    # then its first stage is never filled and every wait is limited to about
    # a millisecond: the waits run out, the call returns the count, and the
    # device stays usable
    import ctypes
    from hamiltonian_diagonalization_gb300 import _capi as C
    torch = cuda
    H, _ = setup(11, 31, 0, ed.odd_coulomb_list(31))
    n = H.GetDimension()
    xd = torch.from_numpy(np.random.default_rng(15).uniform(-1, 1, n)).cuda()
    y6, y7 = torch.empty_like(xd), torch.empty_like(xd)
    H.m_crsSparseMatrix.multiply(xd, y6, 6)
    H.m_crsSparseMatrix.multiply(xd, y7, 7)
    torch.cuda.synchronize()
    assert torch.equal(y6, y7)
    yt = torch.zeros_like(xd)
    timeouts = ctypes.c_int(0)
    C.check(C.lib().ed_spmv_staged_wait_test(H.m_crsSparseMatrix._h, ctypes.c_void_p(xd.data_ptr()),
                                             ctypes.c_void_p(yt.data_ptr()), 2_000_000, ctypes.byref(timeouts)))
    assert timeouts.value >= 16                    # every consumer warp of the stalled CTA
    assert torch.isnan(yt[:16]).all()              # the rows of the never-filled stage
    y7b = torch.empty_like(xd)
    H.m_crsSparseMatrix.multiply(xd, y7b, 7)
    torch.cuda.synchronize()
    assert torch.equal(y7b, y6)
