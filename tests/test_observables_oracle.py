"""The oracle's observables (fermion_observables.hpp restated) pinned by
identities the reference's definitions imply: sum rules, the Lz-reflection
symmetry of a non-degenerate Lz = 0 eigenstate, and the exactly uniform
density of the Laughlin state (V1 only at 2S = 3(N-1): zero energy, total
angular momentum L = 0).  CPU only."""
import numpy as np
import scipy.sparse as sp


def eigenstates(oracle, N, norb, tlz, pp, k=3):
    kt, vt = oracle.quartic_tables(norb, pp)
    b = oracle.basis(N, norb, tlz)
    rp, c, v = oracle.build_upper(b, norb, kt, vt)
    fr, fc, fv = oracle.upper_to_full(rp, c, v, len(b))
    w, vec = np.linalg.eigh(sp.csr_matrix((fv, fc, fr), shape=(len(b), len(b))).toarray())
    return b, w[:k], vec[:, :k].T


def test_sum_rules(oracle):
    N, norb = 5, 13
    b, _, vecs = eigenstates(oracle, N, norb, 3, oracle.odd_coulomb_list(norb))
    for psi in vecs:
        rho = oracle.density(b, psi, norb)
        D = oracle.density_density(b, psi, norb)
        assert abs(rho.sum() - N) < 1e-12                        # particle number
        assert np.allclose(np.diag(D), rho, atol=1e-14)         # n_k^2 = n_k
        assert np.allclose(D, D.T, atol=0)                      # symmetric
        assert np.allclose(D.sum(axis=1), N * rho, atol=1e-12)   # sum_q n_k n_q = N n_k
        pr = oracle.participation_ratio(psi)
        assert 1.0 <= pr <= len(b) + 1e-9


def test_reflection_symmetry_at_lz_zero(oracle):
    # Lz -> -Lz maps orbital k to norb-1-k and the sector to itself
    N, norb = 4, 12
    b, w, vecs = eigenstates(oracle, N, norb, 0, oracle.odd_coulomb_list(norb))
    assert w[1] - w[0] > 1e-6                                    # non-degenerate ground state
    rho = oracle.density(b, vecs[0], norb)
    assert np.allclose(rho, rho[::-1], atol=1e-12)


def test_laughlin_density_is_uniform(oracle):
    for N in (3, 4, 5):
        norb = 3 * (N - 1) + 1
        pp = [0.0, 1.0]                                          # V1 only
        b, w, vecs = eigenstates(oracle, N, norb, 0, pp, k=1)
        assert abs(w[0]) < 1e-12
        rho = oracle.density(b, vecs[0], norb)
        assert np.allclose(rho, N / norb, atol=1e-12), rho


def test_most_probable_order_and_ties(oracle):
    words = np.array([3, 5, 6, 9, 10], dtype=np.uint64)
    psi = np.array([0.1, -0.5, 0.5, 0.2, -0.3])
    s, a = oracle.most_probable(words, psi, 3)
    assert list(s) == [5, 6, 10] and list(a) == [-0.5, 0.5, -0.3]   # |0.5| tie: lower row first
    s, a = oracle.most_probable(words, psi, 10)
    assert len(s) == 5
