"""Two-Landau-level path on the device against the oracle's restatement of
TwoLevelFermionFockBasis and of the two-level Add_CdC / Add_CdCdCC terms:
basis words and ranks exact, CRS bit-exact (upper and full storage, with and
without occupation energies), lowest eigenvalues within 1e-10 relative."""
import numpy as np
import pytest

import hamiltonian_diagonalization_gb300 as ed
from hamiltonian_diagonalization_gb300 import _capi

pytestmark = pytest.mark.gpu

# (N, norb0, 2Lz): integer and half-integer flux, |Lz| > 0, one level empty
# of a sector's states, the largest norb0 the 48-bit words allow
CASES = [(2, 3, 0), (3, 5, 0), (3, 5, 2), (4, 6, 0), (4, 6, -2), (5, 6, 1), (5, 7, 0), (6, 7, 4), (6, 9, 0),
         (4, 23, 0), (2, 23, -20)]


def tables(oracle, norb0, seed):
    rng = np.random.default_rng(seed)
    t0 = ed.QuarticTermTables(norb0, oracle.odd_coulomb_list(norb0))
    t1 = ed.QuarticTermTables(norb0 + 2, rng.uniform(-1.0, 2.0, norb0 + 1))
    return t0, t1


def build(N, norb0, tlz, t0, t1, e0=None, e1=None, upper=True):
    H = ed.TwoLevelSpinlessFermionHamiltonian()
    H.Initialize(N, 2 * norb0 + 2, twoLz=tlz)
    if e0 is not None:
        H.Add_CdC_Terms(e0, 0, 0)
    if e1 is not None:
        H.Add_CdC_Terms(e1, 1, 1)
    H.Add_CdCdCC_Terms(t0, 0, 0, 0, 0, store_upper=upper)
    H.Add_CdCdCC_Terms(t1, 1, 1, 1, 1, store_upper=upper)
    H.Build()
    return H


@pytest.mark.parametrize("case", CASES + [(7, 9, 1)])
def test_basis_and_ranks_exact(cuda, oracle, case):
    N, norb0, tlz = case
    B = ed.TwoLevelFermionFockBasis()
    empty = B.GenerateFockSpace(N, norb0, norb0 + 2, tlz)
    f, s = oracle.basis2(N, norb0, tlz)
    assert empty == (len(f) == 0)
    assert B.GetStoredDimension() == len(f)
    if not len(f):
        return
    df, ds = B.GetFockBasis()
    assert np.array_equal(df, f) and np.array_equal(ds, s)
    for i in range(0, len(f), max(1, len(f) // 50)):
        assert B.FindFockStateIndex(0, int(f[i]), int(s[i])) == i
    # a word with one particle more or fewer is absent
    assert B.FindFockStateIndex(0, int(f[0]), int(s[0]) ^ 1) == _capi.MISS


@pytest.mark.parametrize("case", CASES)
def test_upper_crs_bit_exact(cuda, oracle, case):
    N, norb0, tlz = case
    t0, t1 = tables(oracle, norb0, 3 * norb0 + N)
    f, s = oracle.basis2(N, norb0, tlz)
    rng = np.random.default_rng(N)
    e0 = rng.uniform(-0.5, 0.5, norb0)
    e1 = 1.3 + rng.uniform(-0.5, 0.5, norb0 + 2)
    e1[1] = 0.0                                          # a filtered term
    for energies in ((None, None), (e0, e1)):
        H = build(N, norb0, tlz, t0, t1, *energies, upper=True)
        rp, col, val = H.m_crsSparseMatrix.to_host()
        orp, ocol, oval = oracle.build_upper2(f, s, norb0, t0.m_kTable, t0.m_vTable, t1.m_kTable, t1.m_vTable,
                                              *energies)
        assert np.array_equal(rp, orp)
        assert np.array_equal(col, ocol)
        assert np.array_equal(val.view(np.uint64), oval.view(np.uint64))


@pytest.mark.parametrize("case", [(4, 6, 0), (6, 9, 0), (4, 23, 0)])
def test_full_crs_is_exact_symmetric_completion(cuda, oracle, case):
    N, norb0, tlz = case
    t0, t1 = tables(oracle, norb0, 5)
    e0, e1 = np.linspace(-0.2, 0.2, norb0), np.full(norb0 + 2, 0.7)
    f, s = oracle.basis2(N, norb0, tlz)
    H = build(N, norb0, tlz, t0, t1, e0, e1, upper=False)
    rp, col, val = H.m_crsSparseMatrix.to_host()
    up = oracle.build_upper2(f, s, norb0, t0.m_kTable, t0.m_vTable, t1.m_kTable, t1.m_vTable, e0, e1)
    orp, ocol, oval = oracle.upper_to_full(*up, len(f))
    assert np.array_equal(rp, orp)
    assert np.array_equal(col, ocol)
    assert np.array_equal(val.view(np.uint64), oval.view(np.uint64))


def test_empty_second_level_reduces_to_one_level(cuda, oracle):
    """With no second-level interaction and its orbitals lifted by E = 100, the
    lowest states are the single-level sector's (N=5, 2S=8, Lz=0)."""
    N, norb0 = 5, 9
    pp = oracle.odd_coulomb_list(norb0)
    model = ed.SphereTwoLevelPseudopotentialModel(N, norb0, pp, np.zeros(norb0 + 1), nbrEigenvalues=4)
    model.SetSector(0)
    model.BuildTermTables()
    model.SetOccupationEnergies(np.r_[np.zeros(norb0), np.full(norb0 + 2, 100.0)])
    assert not model.BuildFockBasis()
    model.BuildHamiltonian(store_upper=True)
    assert model.Diagonalize(tol=1e-12, seed=7)
    one = ed.SpinlessFermionHamiltonian()
    one.Initialize(N, norb0, twoLz=0)
    one.Add_CdCdCC_Terms(ed.QuarticTermTables(norb0, pp), store_upper=True)
    one.LanczosDiagonalize(4, tol=1e-12, seed=7)
    assert np.allclose(model.hamiltonian.m_eigenvalues, one.m_eigenvalues, rtol=0, atol=1e-10)


@pytest.mark.parametrize("case,nev", [((6, 9, 0), 6), ((5, 7, 0), 8), ((6, 7, 4), 5)])
def test_lowest_eigenvalues_with_degenerate_copies(cuda, oracle, case, nev):
    """The levels do not mix, so sector eigenvalues E0(L0) + E1(L1) repeat
    2 min(L0, L1) + 1 times; the dense oracle spectrum counts every copy."""
    N, norb0, tlz = case
    t0, t1 = tables(oracle, norb0, 11)
    e0, e1 = np.zeros(norb0), np.full(norb0 + 2, 0.4)
    f, s = oracle.basis2(N, norb0, tlz)
    rp, col, val = oracle.build_upper2(f, s, norb0, t0.m_kTable, t0.m_vTable, t1.m_kTable, t1.m_vTable, e0, e1)
    import scipy.sparse as sp
    A = sp.csr_matrix((val, col, rp), shape=(len(f), len(f)))
    A = (A + sp.triu(A, 1).T).toarray()
    w = np.linalg.eigvalsh(A)[:nev]
    H = build(N, norb0, tlz, t0, t1, e0, e1, upper=True)
    assert H.LanczosDiagonalize(nev, tol=1e-10, seed=3, degeneracy_passes=0)
    scale = max(1.0, float(np.max(np.abs(w))))
    single = H.m_eigenvalues.copy()
    assert np.max(np.abs(single - w)) > 1e-6                       # one sequence misses copies
    assert H.LanczosDiagonalize(nev, tol=1e-10, seed=3, degeneracy_passes=nev), H.last_info
    passes = H.m_eigenvalues.copy()
    assert np.max(np.abs(passes - w)) <= 1e-10 * max(1.0, float(np.max(np.abs(w))))
    assert H.LanczosDiagonalize(nev, tol=1e-10, seed=3), H.last_info   # the ladder, by default
    assert np.max(np.abs(H.m_eigenvalues - w)) <= 1e-10 * scale
    X = np.asarray(H.m_eigenvectors)
    assert np.allclose(X @ X.T, np.eye(nev), atol=1e-8)
    for k in range(nev):
        v = X[k]
        assert np.linalg.norm(A @ v - H.m_eigenvalues[k] * v) <= 1e-9 * scale


def test_mixed_level_terms_refused(cuda, oracle):
    H = ed.TwoLevelSpinlessFermionHamiltonian()
    H.Initialize(3, 12, twoLz=0)
    with pytest.raises(ed.EDError):
        H.Add_CdCdCC_Terms(ed.QuarticTermTables(5, oracle.odd_coulomb_list(5)), 0, 1, 0, 1)
    with pytest.raises(ed.EDError):
        H.Add_CdC_Terms(np.zeros(5), 0, 2)


def test_ladder_solve_refuses_a_one_level_basis(cuda, oracle):
    import ctypes
    one = ed.SpinlessFermionHamiltonian()
    one.Initialize(4, 10, twoLz=0)
    one.Add_CdCdCC_Terms(ed.QuarticTermTables(10, oracle.odd_coulomb_list(10)))
    op = one.operator_handle()
    try:
        p = ed.LanczosParams(nev=2, tol=1e-10)
        ev = np.empty(2)
        st = ed.lib().ed_lanczos_two_level(one.m_fockBasis.handle(), op, ctypes.byref(p), None,
                                           ev.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None, None)
        assert st == _capi.ED_ERR_ARG
    finally:
        ed.lib().ed_op_free(op)


def test_device_crs_matches_reference_build(cuda, oracle):
    # the reference's own two-level model build (its TwoLevelFermionFockBasis
    # and TwoLevelSpinlessFermionHamiltonian compiled from its sources,
    # tests/golden/make_golden_ham.py): same digest of row pointers, columns
    # and FP64 value bits
    import json
    import os
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ref_hamiltonians.json")))
    for key, ent in gold["crs_two_level"].items():
        N, norb0, tlz = ent["N"], ent["norb0"], ent["two_lz"]
        # the term tables the reference run was given (the oracle's)
        kt0, vt0 = oracle.quartic_tables(norb0, oracle.odd_coulomb_list(norb0))
        kt1, vt1 = oracle.quartic_tables(norb0 + 2, oracle.odd_coulomb_list(norb0 + 2))
        t0 = ed.QuarticTermTables(norb0, ktable=kt0, vtable=vt0)
        t1 = ed.QuarticTermTables(norb0 + 2, ktable=kt1, vtable=vt1)
        e0 = np.linspace(-0.3, 0.2, norb0) if ent["energies"] else None
        e1 = np.linspace(0.9, 1.4, norb0 + 2) if ent["energies"] else None
        H = build(N, norb0, tlz, t0, t1, e0, e1, upper=True)
        rp, col, val = H.m_crsSparseMatrix.to_host()
        assert len(rp) - 1 == ent["dim"] and int(rp[-1]) == ent["nnz_upper"], key
        assert oracle.crs_digest(rp, col, val) == ent["sha256"], key


@pytest.mark.parametrize("upper", [False, True])
def test_diagonal_two_level_matrix_from_its_diagonal(cuda, oracle, upper):
    # occupation energies only: the stored matrix is diagonal, and the solve
    # takes the reference's shortcut (MatrixDiagonalCheck) with no product, on
    # the ladder path and the single-sequence path alike
    N, norb0, tlz = 5, 7, 2
    t0 = ed.QuarticTermTables(norb0, np.zeros(norb0 - 1))
    t1 = ed.QuarticTermTables(norb0 + 2, np.zeros(norb0 + 1))
    e0 = np.linspace(-0.3, 0.2, norb0)
    e1 = np.linspace(0.9, 1.4, norb0 + 2)
    H = build(N, norb0, tlz, t0, t1, e0, e1, upper=upper)
    f, s = oracle.basis2(N, norb0, tlz)
    d = np.array([sum(e0[k] for k in range(norb0) if (a >> k) & 1) + sum(e1[k] for k in range(norb0 + 2) if (c >> k) & 1)
                  for a, c in zip(f, s)])
    want = np.sort(d)[:6]
    for passes in (None, 0):
        assert H.LanczosDiagonalize(6, tol=1e-10, seed=2, degeneracy_passes=passes)
        assert H.last_info["matvecs"] == 0
        assert np.max(np.abs(H.m_eigenvalues - want)) <= 1e-12
        V = H.m_eigenvectors
        assert np.allclose(V @ V.T, np.eye(6)) and np.array_equal(np.abs(V).sum(axis=1), np.ones(6))


def test_two_level_product_takes_the_fixed_point_sliced_ell(cuda, oracle):
    # a two-level sector with short rows and more than 4096 of them: the
    # default product is the fixed-point sliced ELL, bit-identical to the
    # fixed-point row kernel (both round each row's exact sum once) and within
    # 1e-13 of the FP64 kernels
    torch = cuda
    t0, t1 = tables(oracle, 11, 31)
    H = build(6, 11, 0, t0, t1, upper=False)    # 6,902 states
    crs = H.m_crsSparseMatrix
    n = crs.GetNbrRows()
    assert n >= 4096 and crs.GetNbrNonZeros() < 96 * n
    x = np.random.default_rng(16).uniform(-1, 1, n)
    xd = torch.from_numpy(x).cuda()
    ys = {}
    for kernel in (0, 4, 6, 8):
        y = torch.full_like(xd, np.nan)
        crs.multiply(xd, y, kernel)
        torch.cuda.synchronize()
        ys[kernel] = y
    assert torch.equal(ys[0], ys[8]) and torch.equal(ys[6], ys[8])
    _, _, val = crs.to_host()
    assert torch.max(torch.abs(ys[4] - ys[8])).item() <= 1e-13 * np.abs(val).max() * 50
