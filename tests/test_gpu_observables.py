"""Observables on the device (ed_obs_*) against the oracle's restatement of
fermion_observables.hpp, on eigenvectors from the device solver and on
random vectors of a large sector; determinism; the Laughlin state's uniform
density as a known answer."""
import numpy as np
import pytest

import hamiltonian_diagonalization_gb300 as ed

pytestmark = pytest.mark.gpu


def solved(N, norb, tlz, pp, nev):
    H = ed.SpinlessFermionHamiltonian()
    H.Initialize(N, norb, twoLz=tlz)
    H.Add_CdCdCC_Terms(ed.QuarticTermTables(norb, pp), store_upper=False)
    H.LanczosDiagonalize(nev, tol=1e-10, seed=5)
    return H


def test_eigenvector_observables_match_oracle(cuda, oracle):
    N, norb = 8, 22
    H = solved(N, norb, 0, oracle.odd_coulomb_list(norb), 3)
    words = oracle.basis(N, norb, 0)
    obs = ed.Observables()
    for e in range(3):
        psi = H.m_eigenvectors[e]
        rho = obs.DensityFunction(H, e)
        D = obs.DensityDensityFunction(H, e)
        assert np.allclose(rho, oracle.density(words, psi, norb), rtol=0, atol=1e-13)
        assert np.allclose(D, oracle.density_density(words, psi, norb), rtol=0, atol=1e-13)
        assert abs(obs.GetParticipationRatio(H, e) / oracle.participation_ratio(psi) - 1.0) < 1e-12
        assert abs(rho.sum() - N) < 1e-9
    top = obs.GetMostProbable(H, 25)
    for e, (s, a) in enumerate(top):
        s_ref, a_ref = oracle.most_probable(words, H.m_eigenvectors[e], 25)
        assert np.array_equal(np.abs(a), np.abs(a_ref))
        assert np.array_equal(a, H.m_eigenvectors[e][np.searchsorted(words, s)])   # each amplitude is its word's


def test_large_sector_random_vector_and_determinism(cuda, oracle):
    N, norb, tlz = 10, 28, 0
    b = ed.FermionFockBasis()
    b.GenerateFockSpace(N, norb, tlz)
    words = oracle.basis(N, norb, tlz)
    rng = np.random.default_rng(17)
    psi = rng.standard_normal(len(words)) * np.exp(rng.uniform(-20, 0, len(words)))
    psi /= np.linalg.norm(psi)
    O = ed.Observables
    rho = O.density_of_vector(b, psi)
    D = O.density_density_of_vector(b, psi)
    assert np.allclose(rho, oracle.density(words, psi, norb), rtol=0, atol=1e-14)
    assert np.allclose(D, oracle.density_density(words, psi, norb), rtol=0, atol=1e-14)
    assert np.array_equal(O.density_of_vector(b, psi).view(np.uint64), rho.view(np.uint64))
    assert np.array_equal(O.density_density_of_vector(b, psi).view(np.uint64), D.view(np.uint64))
    for k in (1, 7, 1000, 100000):
        s, a = O.most_probable_of_vector(b, psi, k)
        s_ref, a_ref = oracle.most_probable(words, psi, k)
        assert np.array_equal(s, s_ref) and np.array_equal(a, a_ref), k


def test_most_probable_ties_and_counts(cuda, oracle):
    N, norb, tlz = 4, 10, 0
    b = ed.FermionFockBasis()
    b.GenerateFockSpace(N, norb, tlz)
    words = oracle.basis(N, norb, tlz)
    n = len(words)
    psi = np.full(n, 0.25)
    psi[::3] = -0.25                 # every entry ties in |psi|
    psi[5] = 0.5
    for k in (0, 1, 4, n, n + 10):
        s, a = ed.Observables.most_probable_of_vector(b, psi, k)
        s_ref, a_ref = oracle.most_probable(words, psi, k)
        assert len(s) == min(k, n)
        assert np.array_equal(s, s_ref) and np.array_equal(a, a_ref), k


def test_laughlin_density_is_uniform(cuda):
    N = 6
    norb = 3 * (N - 1) + 1
    H = solved(N, norb, 0, [0.0, 1.0], 1)
    assert abs(H.m_eigenvalues[0]) < 1e-9
    rho = ed.Observables().DensityFunction(H, 0)
    assert np.allclose(rho, N / norb, atol=1e-8), rho


def test_observables_match_reference(cuda, oracle):
    # the reference's own Observables compiled from its sources
    # (tests/golden/make_golden_ham.py): real seeded vectors for the
    # reductions, complex ones for the most probable states
    import json
    import os
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "ref_hamiltonians.json")))
    o = g["observables"]
    b = ed.FermionFockBasis()
    b.GenerateFockSpace(o["N"], o["norb"], o["two_lz"])
    n = b.GetStoredDimension()
    rng = np.random.default_rng(o["seed"])
    ev = rng.standard_normal((o["nev"], n))
    ev /= np.linalg.norm(ev, axis=1, keepdims=True)
    for e, ref in enumerate(o["vectors"]):
        assert np.max(np.abs(ed.Observables.density_of_vector(b, ev[e]) - ref["density"])) <= 1e-13
        dd = ed.Observables.density_density_of_vector(b, ev[e]).ravel()
        assert np.max(np.abs(dd - np.array(ref["density_density"]))) <= 1e-13
        pr = ed.Observables.participation_ratio_of_vector(b, ev[e])
        assert abs(pr - ref["participation_ratio"]) <= 1e-13 * ref["participation_ratio"]
    m = g["most_probable"]
    bm = ed.FermionFockBasis()
    bm.GenerateFockSpace(m["N"], m["norb"], m["two_lz"])
    n = bm.GetStoredDimension()
    rng = np.random.default_rng(m["seed"])
    v = rng.standard_normal((m["nev"], n))
    v = v + 1j * rng.standard_normal((m["nev"], n))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    k = m["k"]
    states = np.array(m["states"], dtype=np.uint64).reshape(m["nev"], k)
    amps = (np.array(m["amplitudes_re"]) + 1j * np.array(m["amplitudes_im"])).reshape(m["nev"], k)
    for e in range(m["nev"]):
        s, a = ed.Observables.most_probable_of_vector(bm, v[e], k)
        assert np.array_equal(s, states[e])
        assert np.max(np.abs(a - amps[e])) <= 1e-15
