"""Device Lanczos against the eigenvalue oracle (SciPy's ARPACK on the
oracle's matrix, dense LAPACK for small cases) and known answers.
Eigenvalues to 1e-10 relative, residuals ||Hx - lambda x|| <= 1e-10."""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

import hamiltonian_diagonalization_gb300 as ed

pytestmark = pytest.mark.gpu


def model(N, norb, tlz, pp, nev, **kw):
    m = ed.SpherePseudopotentialModel(N, norb, pp, nev)
    m.SetSector(tlz)
    m.BuildTermTables()
    assert m.BuildFockBasis() is False
    m.BuildHamiltonian(matrix_free=kw.pop("matrix_free", False), store_upper=kw.pop("store_upper", False))
    ok = m.Diagonalize(**kw)
    return m, ok


def test_small_config_matches_arpack(cuda, oracle):
    # N=8, 2S=21, Lz=0: 8,512 states, lowest 5, tol 1e-12, seeded start
    N, norb = 8, 22
    pp = oracle.odd_coulomb_list(norb)
    b = oracle.basis(N, norb, 0)
    v0 = oracle.start_vector(len(b), 42)
    kt, vt = oracle.quartic_tables(norb, pp)
    rp, c, v = oracle.build_upper(b, norb, kt, vt)
    wref, _ = oracle.lowest_eigenpairs(rp, c, v, 5, tol=1e-12, v0=v0)
    for kw in ({}, {"store_upper": True}, {"matrix_free": True}):
        m, ok = model(N, norb, 0, pp, 5, tol=1e-10, v0=v0, **kw)
        assert ok, m.hamiltonian.last_info
        w = m.hamiltonian.m_eigenvalues
        assert np.max(np.abs(w - wref) / np.abs(wref)) <= 1e-10, (w, wref)
        info = m.hamiltonian.last_info
        assert info["max_residual"] <= 1e-10 and info["converged"] == 5
        X = m.hamiltonian.m_eigenvectors
        for i in range(5):
            r = oracle.spmv_sym_upper(rp, c, v, X[i]) - w[i] * X[i]
            assert np.linalg.norm(r) <= 1e-10
        assert np.max(np.abs(X @ X.T - np.eye(5))) < 1e-10


def test_sweep_sector_matches_arpack(cuda, oracle):
    N, norb = 10, 28
    pp = oracle.sweep_list(norb, 0.9)
    b = oracle.basis(N, norb, 4)
    kt, vt = oracle.quartic_tables(norb, pp)
    rp, c, v = oracle.build_upper(b, norb, kt, vt)
    fr, fc, fv = oracle.upper_to_full(rp, c, v, len(b))
    A = sp.csr_matrix((fv, fc, fr), shape=(len(b), len(b)))
    import scipy.sparse.linalg as sla
    v0 = oracle.start_vector(len(b), 3)
    wref = np.sort(sla.eigsh(A, k=4, which="SA", tol=1e-13, v0=v0)[0])
    m, ok = model(N, norb, 4, pp, 4, tol=1e-10, v0=v0)
    assert ok
    w = m.hamiltonian.m_eigenvalues
    assert np.max(np.abs(w - wref) / np.abs(wref)) <= 1e-10


def test_two_particle_and_laughlin_known_answers(cuda):
    # N=2: levels are 2*V_m (the reference's normalisation); 2S = 9 -> 10 orbitals
    pp = [0.0, 1.3, 0.0, 0.7, 0.0, 0.25, 0.0, 0.1, 0.0]
    m, ok = model(2, 10, 0, pp, 4, tol=1e-12)
    assert ok
    assert np.allclose(m.hamiltonian.m_eigenvalues, [0.0, 0.2, 0.5, 1.4], atol=1e-12)
    # V1 only at 2S = 3(N-1): the Laughlin state has exactly zero energy
    m, ok = model(6, 16, 0, [0.0, 1.0], 2, tol=1e-11)
    assert ok
    assert abs(m.hamiltonian.m_eigenvalues[0]) < 1e-10 and m.hamiltonian.m_eigenvalues[1] > 1e-3


def test_host_callback_operator_and_dense_path(cuda, oracle):
    # std::function form: a host matvec; n < 60 goes through the dense path
    for n in (40, 300):
        rng = np.random.default_rng(n)
        Q = np.linalg.qr(rng.standard_normal((n, n)))[0]
        d = np.sort(rng.uniform(-3, 5, n))
        A = (Q * d) @ Q.T
        arp = ed.ArpackWrapper()
        ev = np.empty(3)
        vec = np.empty((3, n))
        ok = arp.DiagonalizeSymmetricMatrix(lambda x, y: np.copyto(y, A @ x), vec, ev, n, n, 3, tol=1e-11)
        assert ok, arp.last_info
        assert np.allclose(ev, d[:3], atol=1e-10)


def test_breakdown_in_invariant_subspace(cuda):
    # A diagonal operator with 4 distinct eigenvalues: the Krylov space is
    # exhausted after 4 steps and the solver must restart with fresh vectors
    n = 500
    d = np.repeat([-2.0, -1.0, 0.5, 3.0], n // 4)
    arp = ed.ArpackWrapper()
    ev = np.empty(3)
    ok = arp.DiagonalizeSymmetricMatrix(lambda x, y: np.multiply(d, x, out=y), None, ev, n, n, 3, tol=1e-10,
                                        v0=np.ones(n))
    assert ok, arp.last_info
    assert arp.last_info["breakdowns"] >= 1
    assert np.allclose(ev, [-2.0, -2.0, -2.0], atol=1e-10)


def test_degeneracy_passes_recover_copies(cuda):
    """A random rotation of a spectrum with a 3-fold and a 2-fold lowest pair
    of values, through a host operator: the deflated passes return every copy
    with orthonormal vectors.  (Here rounding in the dense product already
    lets one Krylov sequence find the copies; the two-level tests hold
    sectors where it does not.)"""
    n, nev = 400, 6
    rng = np.random.default_rng(5)
    d = np.sort(np.r_[[-3.0] * 3, [-2.5] * 2, rng.uniform(-2.0, 4.0, n - 5)])
    Q = np.linalg.qr(rng.standard_normal((n, n)))[0]
    A = (Q * d) @ Q.T
    A = 0.5 * (A + A.T)

    def solve(passes):
        arp = ed.ArpackWrapper()
        ev, vec = np.empty(nev), np.empty((nev, n))
        assert arp.DiagonalizeSymmetricMatrix(lambda x, y: np.copyto(y, A @ x), vec, ev, n, n, nev, tol=1e-10,
                                              seed=1, degeneracy_passes=passes), arp.last_info
        return ev, vec, arp.last_info

    ev, vec, info = solve(nev)
    assert np.allclose(ev, d[:nev], atol=1e-10)
    assert np.allclose(vec @ vec.T, np.eye(nev), atol=1e-8)
    assert np.max(np.linalg.norm(vec @ A - ev[:, None] * vec, axis=1)) <= 1e-9
    assert info["converged"] == nev


def test_no_convergence_reported(cuda, oracle):
    N, norb = 8, 22
    H = ed.SpinlessFermionHamiltonian()
    H.Initialize(N, norb, twoLz=0)
    H.Add_CdCdCC_Terms(ed.QuarticTermTables(norb, oracle.odd_coulomb_list(norb)))
    ok = H.LanczosDiagonalize(5, tol=1e-30, max_restarts=1)
    assert ok is False
    assert H.last_info["restarts"] == 1
    # the best Ritz values so far are still returned and are close
    assert np.all(np.isfinite(H.m_eigenvalues))


def test_bad_start_vector_rejected(cuda):
    for (N, norb) in [(4, 12), (6, 16)]:      # dense path (dim < 60) and Lanczos path
        H = ed.SpinlessFermionHamiltonian()
        H.Initialize(N, norb, twoLz=0)
        H.Add_CdCdCC_Terms(ed.QuarticTermTables(norb, [0.0, 1.0]))
        n = H.GetDimension()
        assert H.LanczosDiagonalize(2, v0=np.zeros(n)) is False
        bad = np.ones(n)
        bad[3] = np.nan
        assert H.LanczosDiagonalize(2, v0=bad) is False
        assert H.LanczosDiagonalize(2, v0=np.ones(n)) is True


def test_one_call_solve_matches_stepwise(cuda, oracle):
    N, norb = 8, 22
    pp = oracle.odd_coulomb_list(norb)
    n = len(oracle.basis(N, norb, 0))
    v0 = oracle.start_vector(n, 42)
    out = ed.solve_sector(N, norb, 0, pp, 5, tol=1e-10, v0=v0, want_vectors=True)
    m, ok = model(N, norb, 0, pp, 5, tol=1e-10, v0=v0)
    assert np.max(np.abs(out["eigenvalues"] - m.hamiltonian.m_eigenvalues)) <= 1e-11
    assert out["info"]["max_residual"] <= 1e-10
    out2 = ed.solve_sector(N, norb, 0, pp, 5, tol=1e-10, v0=v0, matrix_free=True)
    assert np.max(np.abs(out2["eigenvalues"] - out["eigenvalues"])) <= 1e-11


def test_stored_crs_config_matches_arpack_fixture(cuda):
    # N=11, 2S=30, Lz=0 (1,371,535 states): the 10 lowest eigenvalues against
    # the reference-family ARPACK run recorded in tests/golden
    import json
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "arpack_n11_2s30_lz0.json")
    if not os.path.exists(path):
        pytest.skip("ARPACK fixture not generated yet (tests/golden/make_arpack_fixture.py)")
    ref = json.load(open(path))
    n = ref["n"]
    v0 = np.random.default_rng(ref["seed"]).uniform(-1.0, 1.0, n)
    v0 /= np.linalg.norm(v0)
    out = ed.solve_sector(ref["N"], ref["norb"], ref["two_lz"], ed.odd_coulomb_list(ref["norb"]), ref["nev"],
                          tol=1e-10, v0=v0)
    w = out["eigenvalues"]
    wref = np.array(ref["eigenvalues"])
    assert np.max(np.abs(w - wref) / np.abs(wref)) <= 1e-10, (w, wref)
    assert out["info"]["max_residual"] <= 1e-10
