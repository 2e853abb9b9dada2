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
    # every full-storage kernel (row lanes, shared-reduction rows, sliced ELL) on every sector,
    # including ones with fewer rows than a tile and with empty rows
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
    for kernel in range(1, 6):
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
