"""Complex momentum path on the device (optical-flux-lattice model) against
the oracle's restatement of the momentum basis and of
SpinlessFermionHamiltonian<dcmplx>: basis words and ranks exact, complex CRS
bit-exact in upper (the reference's) and full storage, products to 1e-13,
eigenvalues to 1e-10 of dense spectra, residuals to 1e-9."""
import numpy as np
import pytest
import scipy.sparse as sp

import hamiltonian_diagonalization_gb300 as ed
from hamiltonian_diagonalization_gb300 import _capi

pytestmark = pytest.mark.gpu

# grids down to one column or row, and the 40-orbital limit (5 x 8)
CASES = [(3, 3, 4, 0, 0), (4, 3, 4, 1, 2), (5, 3, 4, 2, 3), (6, 4, 4, 0, 1), (5, 4, 5, 3, 2), (4, 4, 6, 1, 5),
         (4, 1, 9, 0, 4), (3, 8, 1, 5, 0), (3, 5, 8, 2, 5)]


def tables(oracle, X, Y, seed):
    kt, vt = oracle.ofl_tables(X, Y, seed)
    return ed.ComplexQuarticTermTables(X, Y, kt, vt)


def build(N, X, Y, kx, ky, T, energies=None, upper=True):
    model = ed.InteractingOflModel(N, X, Y, T, energies)
    model.SetSector(kx, ky)
    empty = model.BuildFockBasis()
    if not empty:
        model.BuildHamiltonian(store_upper=upper)
    return model, empty


@pytest.mark.parametrize("case", CASES + [(2, 1, 3, 0, 2), (7, 4, 5, 3, 4)])
def test_momentum_basis_and_ranks_exact(cuda, oracle, case):
    N, X, Y, kx, ky = case
    B = ed.FermionFockBasis()
    empty = B.GenerateFockSpaceMomentum(N, X, Y, kx, ky)
    b = oracle.basis_momentum(N, X, Y, kx, ky)
    assert empty == (len(b) == 0)
    assert B.GetStoredDimension() == len(b)
    if len(b):
        assert np.array_equal(B.GetFockBasis(), b)
        idx = B.FindFockStateIndices(b)
        assert np.array_equal(idx, np.arange(len(b), dtype=np.uint64))
        assert B.FindFockStateIndex(0, int(b[0]) ^ 1) == _capi.MISS


@pytest.mark.parametrize("case", CASES)
def test_complex_crs_bit_exact(cuda, oracle, case):
    N, X, Y, kx, ky = case
    K = X * Y
    T = tables(oracle, X, Y, K + N)
    b = oracle.basis_momentum(N, X, Y, kx, ky)
    e = np.linspace(-0.4, 0.6, K) + 1e-3j * np.arange(K)
    e[2] = 0.0                                         # a filtered term
    for energies in (None, e):
        model, _ = build(N, X, Y, kx, ky, T, energies, upper=True)
        rp, col, val = model.hamiltonian.m_crsSparseMatrix.to_host()
        orp, ocol, oval = oracle.build_upper_complex(b, K, T.m_kTable, T.m_vTable, energies)
        assert np.array_equal(rp, orp)
        assert np.array_equal(col, ocol)
        assert np.array_equal(val.view(np.uint64), oval.view(np.uint64))
        full, _ = build(N, X, Y, kx, ky, T, energies, upper=False)
        frp, fcol, fval = full.hamiltonian.m_crsSparseMatrix.to_host()
        mrp, mcol, mval = oracle.complex_upper_to_full(orp, ocol, oval, len(b))
        assert np.array_equal(frp, mrp) and np.array_equal(fcol, mcol)
        assert np.array_equal(fval.view(np.uint64), mval.view(np.uint64))


@pytest.mark.parametrize("case", [(5, 3, 4, 2, 3), (5, 4, 5, 3, 2)])
def test_complex_products(cuda, oracle, case):
    torch = cuda
    N, X, Y, kx, ky = case
    K = X * Y
    T = tables(oracle, X, Y, 11)
    b = oracle.basis_momentum(N, X, Y, kx, ky)
    orp, ocol, oval = oracle.build_upper_complex(b, K, T.m_kTable, T.m_vTable)
    mrp, mcol, mval = oracle.complex_upper_to_full(orp, ocol, oval, len(b))
    M = sp.csr_matrix((mval, mcol, mrp), shape=(len(b), len(b)))
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, len(b)) + 1j * rng.uniform(-1, 1, len(b))
    yref = M @ x
    scale = np.abs(oval).max() * 50
    for upper in (True, False):
        model, _ = build(N, X, Y, kx, ky, T, upper=upper)
        xd = torch.from_numpy(x.view(np.float64).copy()).cuda()
        yd = torch.empty_like(xd)
        model.hamiltonian.apply(xd, yd)
        torch.cuda.synchronize()
        y = yd.cpu().numpy().view(np.complex128)
        assert np.max(np.abs(y - yref)) <= 1e-13 * scale


@pytest.mark.parametrize("case,nev", [((3, 3, 4, 0, 0), 3), ((5, 3, 4, 2, 3), 4), ((6, 4, 4, 0, 1), 5),
                                      ((5, 4, 5, 3, 2), 6), ((4, 4, 6, 1, 5), 4)])
def test_complex_eigenpairs(cuda, oracle, case, nev):
    N, X, Y, kx, ky = case
    K = X * Y
    T = tables(oracle, X, Y, 5)
    e = np.linspace(-0.2, 0.3, K)
    b = oracle.basis_momentum(N, X, Y, kx, ky)
    orp, ocol, oval = oracle.build_upper_complex(b, K, T.m_kTable, T.m_vTable, e)
    M = sp.csr_matrix(oracle.complex_upper_to_full(orp, ocol, oval, len(b))[::-1], shape=(len(b), len(b)))
    A = M.toarray()
    w = np.linalg.eigvalsh(A)[:nev]
    for upper in (False, True):
        model, _ = build(N, X, Y, kx, ky, T, e, upper=upper)
        model.nev = nev
        assert model.Diagonalize(tol=1e-10, seed=2), model.hamiltonian.last_info
        H = model.hamiltonian
        scale = max(1.0, float(np.abs(w).max()))
        assert np.max(np.abs(H.m_eigenvalues - w)) <= 1e-10 * scale
        X_ = H.m_eigenvectors
        assert np.allclose(X_.conj() @ X_.T, np.eye(nev), atol=1e-8)
        for k in range(nev):
            assert np.linalg.norm(A @ X_[k] - H.m_eigenvalues[k] * X_[k]) <= 1e-9 * scale


def test_complex_solver_through_breakdowns(cuda, oracle):
    # no interaction and energies k mod 3: H is diagonal with a handful of
    # distinct, highly degenerate values, so every Krylov sequence breaks
    # down after a few steps and each degenerate copy needs a fresh direction
    N, X, Y, kx, ky = 6, 4, 4, 0, 1
    K = X * Y
    kt, vt = oracle.ofl_tables(X, Y, 5)
    T = ed.ComplexQuarticTermTables(X, Y, kt, np.zeros_like(vt))
    e = (np.arange(K) % 3).astype(float)
    b = oracle.basis_momentum(N, X, Y, kx, ky)
    orp, ocol, oval = oracle.build_upper_complex(b, K, T.m_kTable, T.m_vTable, e)
    A = oracle.complex_upper_to_full(orp, ocol, oval, len(b))
    w = np.linalg.eigvalsh(sp.csr_matrix(A[::-1], shape=(len(b), len(b))).toarray())
    nev = 8
    assert w[nev - 1] == w[0]          # the lowest value alone has more than nev copies
    for upper in (False, True):
        model, _ = build(N, X, Y, kx, ky, T, e, upper=upper)
        model.nev = nev
        # the Krylov path itself (the diagonal shortcut off)
        assert model.Diagonalize(tol=1e-10, seed=3, diagonal_check=False), model.hamiltonian.last_info
        H = model.hamiltonian
        assert H.last_info["breakdowns"] >= 1
        assert np.max(np.abs(H.m_eigenvalues - w[:nev])) <= 1e-10
        X_ = H.m_eigenvectors
        assert np.allclose(X_.conj() @ X_.T, np.eye(nev), atol=1e-8)


def test_lz_build_refuses_a_momentum_basis(cuda):
    B = ed.FermionFockBasis()
    B.GenerateFockSpaceMomentum(3, 3, 4, 0, 0)
    H = ed.SpinlessFermionHamiltonian()
    H.m_fockBasis = B
    with pytest.raises(ed.EDError):
        H.Add_CdCdCC_Terms(ed.QuarticTermTables(12, [0.0, 1.0]))


def test_tables_that_break_momentum_are_refused(cuda, oracle):
    kt, vt = oracle.ofl_tables(3, 4, 1)
    kt = kt.copy()
    i = oracle.ofl_index(0, 1, 12) * 12 + 5             # k3 = 0, k4 = 1, k2 = 5
    kt[i] = (int(kt[i]) + 1) % 12
    T = ed.ComplexQuarticTermTables(3, 4, kt, vt)
    model = ed.InteractingOflModel(3, 3, 4, T)
    model.SetSector(0, 0)
    model.BuildFockBasis()
    with pytest.raises(ed.EDError):
        model.BuildHamiltonian()


def test_observables_of_complex_eigenvectors(cuda, oracle):
    """fermion_observables.hpp on the model's complex eigenvectors: density,
    density-density and participation ratio from |psi|, the most probable
    states with their complex amplitudes."""
    N, X, Y, kx, ky = 5, 4, 5, 3, 2
    T = tables(oracle, X, Y, 5)
    model, _ = build(N, X, Y, kx, ky, T, upper=False)
    model.nev = 2
    assert model.Diagonalize(tol=1e-10, seed=2)
    H = model.hamiltonian
    words = H.m_fockBasis.GetFockBasis()
    psi = H.m_eigenvectors[0]
    assert np.iscomplexobj(psi) and np.abs(psi.imag).max() > 1e-3
    obs = ed.Observables()
    K = X * Y
    mag = np.abs(psi)
    assert np.allclose(obs.DensityFunction(H, 0), oracle.density(words, mag, K), atol=1e-13)
    assert np.allclose(obs.DensityDensityFunction(H, 0), oracle.density_density(words, mag, K), atol=1e-13)
    assert abs(obs.GetParticipationRatio(H, 0) - oracle.participation_ratio(mag)) <= 1e-10 * len(words)
    states, amps = ed.Observables.most_probable_of_vector(H.m_fockBasis, psi, 10)
    ostates, _ = oracle.most_probable(words, mag, 10)
    assert np.array_equal(states, ostates)
    idx = np.searchsorted(words, states)
    assert np.array_equal(amps, psi[idx])


def test_empty_momentum_sector(cuda, oracle):
    """A sector with no states: N=3 on a 1x3 grid has one word, whose ky sum
    0+1+2 is 0 mod 3, so the sector ky = 1 is empty.  Building works and the
    solve reports an empty operator."""
    kt, vt = oracle.ofl_tables(1, 3, 0)
    T = ed.ComplexQuarticTermTables(1, 3, kt, vt)
    model = ed.InteractingOflModel(3, 1, 3, T)
    model.SetSector(0, 1)
    assert model.BuildFockBasis() is True
    model.BuildHamiltonian()
    assert model.hamiltonian.m_crsSparseMatrix.GetNbrRows() == 0
    assert model.Diagonalize() is False
    assert "dimension 0" in model.hamiltonian.last_error


def test_device_crs_matches_reference_build(cuda, oracle):
    # the reference's own complex build (its SpinlessFermionHamiltonian<dcmplx>,
    # momentum-sector basis and array-format tables compiled from its sources,
    # tests/golden/make_golden_ham.py): same digest of the device's CRS
    import json
    import os
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ref_hamiltonians.json")))
    for key, ent in gold["crs_complex"].items():
        N, X, Y, kx, ky = ent["N"], ent["X"], ent["Y"], ent["kx"], ent["ky"]
        K = X * Y
        T = tables(oracle, X, Y, K + N)
        e = (np.linspace(-0.4, 0.6, K) + 1e-3j * np.arange(K)) if ent["energies"] else None
        model, empty = build(N, X, Y, kx, ky, T, e, upper=True)
        assert not empty
        rp, col, val = model.hamiltonian.m_crsSparseMatrix.to_host()
        assert len(rp) - 1 == ent["dim"] and int(rp[-1]) == ent["nnz_upper"], key
        assert oracle.crs_digest(rp, col, np.ascontiguousarray(val).view(np.float64)) == ent["sha256"], key


def test_hash_format_build_matches_reference_hash_path(cuda, oracle, tmp_path):
    # hash-table files from this project's writer, built by the reference's own
    # hash path (TermsFromFile + the hash branch of BuildHamiltonian,
    # tests/golden/make_golden_ham.py) and here from the same files: same
    # digest; binary files give the array path's digest, text ones keep 15
    # significant digits
    import json
    import os
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ref_hamiltonians.json")))
    for key, ent in gold["crs_complex_hash"].items():
        N, X, Y, kx, ky, fmt = ent["N"], ent["X"], ent["Y"], ent["kx"], ent["ky"], ent["format"]
        K = X * Y
        kt, vt = oracle.ofl_tables(X, Y, K + N)
        e = (np.linspace(-0.4, 0.6, K) + 1e-3j * np.arange(K)) if ent["energies"] else None
        m = ed.InteractingOflModel(N, X, Y, ed.ComplexQuarticTermTables(X, Y, kt, vt), e)
        m.ConvertTableFormat()
        d = str(tmp_path / key)
        os.makedirs(d)
        m.TermsToFile(d, fmt)
        m2 = ed.InteractingOflModel(N, X, Y, None)
        m2.TermsFromFile(d, fmt)
        m2.SetSector(kx, ky)
        assert not m2.BuildFockBasis()
        m2.BuildHamiltonian(store_upper=True)
        rp, col, val = m2.hamiltonian.m_crsSparseMatrix.to_host()
        assert len(rp) - 1 == ent["dim"] and int(rp[-1]) == ent["nnz_upper"], key
        assert oracle.crs_digest(rp, col, np.ascontiguousarray(val).view(np.float64)) == ent["sha256"], key


def test_hash_build_refuses_what_the_arrays_cannot_hold(cuda, oracle, tmp_path):
    import os
    X, Y, N = 2, 3, 3
    K = X * Y
    kt, vt = oracle.ofl_tables(X, Y, 11)

    def model_with(quartic, quadratic):
        m = ed.InteractingOflModel(N, X, Y, None)
        m.m_tableFormat = "hash"
        m.m_quarticHashTables, m.m_quadraticHashTables = quartic, quadratic
        m.SetSector(0, 0)
        m.BuildFockBasis()
        return m

    T = ed.ComplexQuarticTermTables(X, Y, kt, vt)
    good = ed.QuarticTermHashTables()
    good.SetQuarticFromArray(T)
    diag = ed.QuadraticTermHashTables()
    diag.SetQuadraticFromArray(np.linspace(-0.4, 0.6, K))
    model_with(good, diag).BuildHamiltonian()      # builds
    # the reference's own file lacks the k1 of (0, 0, 1): refused, not read past
    ref = ed.QuarticTermHashTables()
    ref.FromFile(os.path.join(os.path.dirname(__file__), "golden", "ofl_hash_ref_2x3_quartic.bin"), "binary")
    with pytest.raises(ed.EDError):
        model_with(ref, diag).BuildHamiltonian()
    # two k1 for one (k2, k3, k4): not momentum-conserving
    two = ed.QuarticTermHashTables()
    two._set(np.append(good.kkeys, good.kkeys[5]), np.append(good.kvals, (good.kvals[5] + 1) % K),
             good.vkeys, good.vvals)
    with pytest.raises(ed.EDError):
        model_with(two, diag).BuildHamiltonian()
    # an off-diagonal one-body term
    off = ed.QuadraticTermHashTables()
    off._set(diag.kkeys, np.roll(diag.kvals, 1), diag.vkeys, diag.vvals)
    with pytest.raises(ed.EDError):
        model_with(good, off).BuildHamiltonian()
    # two values for one array slot
    bad = ed.QuarticTermHashTables()
    vv = good.vvals.copy()
    k2, k3, k4 = 1, 0, 2                            # k4 > k3: its value sits in slot k1
    k1 = T.GetK1(k2, k3, k4)[0]
    i = int(np.nonzero(good.vkeys == np.uint64(ed.hash_key(k1, k2, k3, k4)))[0][0])
    vv[i] += 0.5
    bad._set(good.kkeys, good.kvals, good.vkeys, vv)
    with pytest.raises(ed.EDError):
        model_with(bad, diag).BuildHamiltonian()


def test_diagonal_matrix_is_solved_from_its_diagonal(cuda, oracle):
    # no interaction: the stored matrix is diagonal, and LanczosDiagonalize
    # takes the reference's shortcut (MatrixDiagonalCheck): the nev lowest
    # diagonal entries, no product, each copy of a repeated value its own
    # unit vector (the reference gives every copy the same one)
    N, X, Y, kx, ky = 6, 4, 4, 0, 1
    K = X * Y
    kt, vt = oracle.ofl_tables(X, Y, 5)
    T = ed.ComplexQuarticTermTables(X, Y, kt, np.zeros_like(vt))
    e = (np.arange(K) % 3).astype(float) + 0.25 * (np.arange(K) % 2)
    b = oracle.basis_momentum(N, X, Y, kx, ky)
    d = np.sort(np.array([sum(e[k] for k in range(K) if (w >> k) & 1) for w in b]))
    for upper in (False, True):
        model, _ = build(N, X, Y, kx, ky, T, e, upper=upper)
        model.nev = 9
        assert model.Diagonalize(tol=1e-10, seed=3)
        H = model.hamiltonian
        assert H.last_info["matvecs"] == 0 and H.last_info["converged"] == 9
        assert np.max(np.abs(H.m_eigenvalues - d[:9])) <= 1e-12
        V = H.m_eigenvectors
        assert np.array_equal(np.abs(V).sum(axis=1), np.ones(9))              # unit vectors
        assert np.allclose(V.conj() @ V.T, np.eye(9))                          # distinct positions


def _fix_ints(v):
    """The fixed-point integers A = round(v 2^(1080 - E)) (nearest, ties away
    from zero) of float64 v and E, the largest biased exponent field (>= 1)."""
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
    return np.where((b >> np.uint64(63)).astype(bool), -q, q), E


def _round(S, sc):
    return S / (1 << -sc) if sc < 0 else float(S << sc)   # one rounding to nearest even


@pytest.mark.parametrize("case", [(5, 3, 4, 2, 3), (4, 4, 6, 1, 5)])
def test_fixed_point_complex_product_is_exactly_rounded(cuda, oracle, case):
    # the integer kernel against the exact integer sums of its fixed-point
    # inputs rounded once, bit for bit; the FP64 kernel to 1e-13
    torch = cuda
    N, X, Y, kx, ky = case
    T = tables(oracle, X, Y, 11)
    model, _ = build(N, X, Y, kx, ky, T, upper=False)
    crs = model.hamiltonian.m_crsSparseMatrix
    rp, col, val = crs.to_host()
    n = len(rp) - 1
    A, ea = _fix_ints(val.view(np.float64))
    rng = np.random.default_rng(7)
    for x in (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n),
              (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * np.exp(rng.uniform(-30, 3, n))):
        Xq, ex = _fix_ints(x.view(np.float64))
        ar, ai = A[0::2].tolist(), A[1::2].tolist()
        xr, xi = Xq[0::2].tolist(), Xq[1::2].tolist()
        sc = ea + ex - 2160
        ref = np.empty(2 * n)
        for i in range(n):
            sre = sim = 0
            for k in range(rp[i], rp[i + 1]):
                c = col[k]
                sre += ar[k] * xr[c] - ai[k] * xi[c]
                sim += ar[k] * xi[c] + ai[k] * xr[c]
            ref[2 * i], ref[2 * i + 1] = _round(sre, sc), _round(sim, sc)
        xd = torch.from_numpy(x.view(np.float64).copy()).cuda()
        y2, y1, y0 = torch.empty_like(xd), torch.empty_like(xd), torch.empty_like(xd)
        crs.multiply(xd, y2, 2)
        crs.multiply(xd, y1, 1)
        model.hamiltonian.apply(xd, y0)
        torch.cuda.synchronize()
        assert np.array_equal(y2.cpu().numpy().view(np.uint64), ref.view(np.uint64))
        assert torch.equal(y0, y2)                     # full storage uses the integer kernel
        scale = np.abs(val).max() * np.abs(x).max() * 50
        assert np.max(np.abs((y1 - y2).cpu().numpy())) <= 1e-13 * scale


def test_fixed_point_complex_product_edges(cuda, oracle):
    torch = cuda
    T = tables(oracle, 3, 4, 11)
    model, _ = build(5, 3, 4, 2, 3, T, upper=False)
    crs = model.hamiltonian.m_crsSparseMatrix
    n = crs.GetNbrRows()
    x = np.random.default_rng(8).uniform(-1, 1, 2 * n)
    x[5] = np.inf
    xd = torch.from_numpy(x).cuda()
    y = torch.zeros_like(xd)
    crs.multiply(xd, y, 2)
    torch.cuda.synchronize()
    assert torch.isnan(y).all()                        # a non-finite entry of x: every entry NaN
    up, _ = build(5, 3, 4, 2, 3, T, upper=True)
    with pytest.raises(ed.EDError):
        up.hamiltonian.m_crsSparseMatrix.multiply(xd, torch.empty_like(xd), 2)
