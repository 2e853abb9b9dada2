"""Known-answer checks of the oracle's Hamiltonian (CPU): these physics
identities pin the sign conventions, the Clebsch-Gordan normalisation and the
indexing of the restated build, since the reference ships no fixtures for
them."""
import numpy as np
import scipy.sparse as sp


def dense(oracle, N, norb, tlz, pp):
    kt, vt = oracle.quartic_tables(norb, pp)
    b = oracle.basis(N, norb, tlz)
    rp, c, v = oracle.build_upper(b, norb, kt, vt)
    fr, fc, fv = oracle.upper_to_full(rp, c, v, len(b))
    return sp.csr_matrix((fv, fc, fr), shape=(len(b), len(b))).toarray()


def test_two_particles_spectrum_is_twice_pseudopotentials(oracle):
    # H = sum_{k1..k4} V c+c+cc with the reference's sign and no 1/2: a pair
    # with relative angular momentum m has energy 2 V_m
    norb = 9
    pp = [0.3, 1.1, 0.0, 0.6, 0.7, 0.2, 0.0, 0.05]
    two_s = norb - 1
    for tlz in (0, 2, 4):
        w = np.linalg.eigvalsh(dense(oracle, 2, norb, tlz, pp))
        # one level per pair momentum J = 2S - m >= |Lz| with m odd (fermions)
        expect = sorted(2.0 * (pp[m] if m < len(pp) else 0.0)
                        for m in range(1, two_s + 1, 2) if two_s - m >= abs(tlz) // 2)
        assert len(w) == len(expect)
        assert np.allclose(sorted(w), expect, atol=1e-12)


def test_laughlin_state_has_zero_energy(oracle):
    for N in (3, 4, 5):
        norb = 3 * (N - 1) + 1
        w = np.linalg.eigvalsh(dense(oracle, N, norb, 0, [0.0, 1.0]))
        assert abs(w[0]) < 1e-12 and w[1] > 1e-3


def test_even_pseudopotentials_do_not_act_on_fermions(oracle):
    a = dense(oracle, 4, 11, 0, [0.0, 1.0, 0.0, 0.4])
    b = dense(oracle, 4, 11, 0, [0.9, 1.0, 2.5, 0.4])
    assert np.allclose(np.linalg.eigvalsh(a), np.linalg.eigvalsh(b), atol=1e-12)


def test_lz_reflection_symmetry(oracle):
    pp = oracle.odd_coulomb_list(12)
    a = np.linalg.eigvalsh(dense(oracle, 4, 12, 4, pp))
    b = np.linalg.eigvalsh(dense(oracle, 4, 12, -4, pp))
    assert np.allclose(a, b, atol=1e-12)


def test_hermitian_and_rotational_multiplets(oracle):
    pp = oracle.odd_coulomb_list(10)
    h0 = dense(oracle, 4, 10, 0, pp)
    assert np.array_equal(h0, h0.T)
    # every Lz=2 level is also an Lz=0 level (L >= 1 multiplets)
    w0 = np.linalg.eigvalsh(h0)
    w1 = np.linalg.eigvalsh(dense(oracle, 4, 10, 2, pp))
    for e in w1:
        assert np.min(np.abs(w0 - e)) < 1e-10


def test_arpack_oracle_agrees_with_dense(oracle):
    pp = oracle.odd_coulomb_list(13)
    b = oracle.basis(5, 13, 0)
    kt, vt = oracle.quartic_tables(13, pp)
    rp, c, v = oracle.build_upper(b, 13, kt, vt)
    fr, fc, fv = oracle.upper_to_full(rp, c, v, len(b))
    H = sp.csr_matrix((fv, fc, fr), shape=(len(b), len(b))).toarray()
    wd = np.linalg.eigvalsh(H)[:4]
    w, vec = oracle.lowest_eigenpairs(rp, c, v, 4, tol=1e-12, v0=oracle.start_vector(len(b), 1))
    assert np.allclose(w, wd, rtol=1e-11, atol=1e-11)
    y = oracle.spmv_sym_upper(rp, c, v, vec[:, 0])
    assert np.linalg.norm(y - w[0] * vec[:, 0]) < 1e-9
