"""Pin the CPU oracle against the reference's own code.

Fixtures in tests/golden/ were produced by the reference's primitives compiled
from its sources (tests/golden/make_golden.py); when that compiled library is
present (oracle/_ref, built only where the reference tree exists) the oracle
is also checked against it on fresh random inputs."""
import hashlib
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def prim():
    return dict(np.load(os.path.join(GOLD, "ref_primitives.npz")))


@pytest.fixture(scope="module")
def bases():
    with open(os.path.join(GOLD, "ref_bases.json")) as f:
        return json.load(f)


def test_evaluate_cdcdcc_matches_reference(oracle, prim):
    rec = prim["cdcdcc"]
    bad = 0
    for norb, k1, k2, k3, k4, state, out, sign2 in rec.astype(object):
        o, s = oracle.evaluate_cdcdcc(int(k1), int(k2), int(k3), int(k4), int(state), int(norb))
        sign = int(sign2) - 2
        if s != sign or (sign != 0 and o != int(out)):
            bad += 1
    assert bad == 0
    # both vanishing and non-vanishing cases are covered
    signs = rec[:, 7].astype(int) - 2
    assert (signs == 0).sum() > 1000 and (signs == 1).sum() > 1000 and (signs == -1).sum() > 1000


def test_hamming_tools_match_reference(oracle, prim):
    for x, nx in prim["next_hamming"].astype(object):
        assert oracle.next_hamming(int(x)) == int(nx)
    for w, idx, val in prim["generate_hamming"].astype(object):
        assert oracle.unrank_hamming(int(w), int(idx)) == int(val)
    for x, c in prim["hamming_weight"].astype(object):
        assert bin(int(x)).count("1") == int(c)
    for x, p in prim["base2log"].astype(object):
        assert int(x).bit_length() - 1 == int(p)


def test_lz_predicate_matches_reference(oracle, prim):
    for state, tlz, maxlz, ok in prim["lz_ok"]:
        assert oracle.lz_ok(int(state), int(tlz), int(maxlz)) == bool(ok)


def test_binomials_match_reference_table(oracle, prim):
    # The reference's table was generated in double precision: entries from
    # about 2e15 up are off by a few units in the last place.  Every binomial
    # the measured configurations use (C(34,12) ~ 5.5e8 and below) is exact.
    for n, k, v in prim["binomial"]:
        exact = oracle.binomial(int(n), int(k))
        if exact < 10 ** 15:
            assert exact == int(v)
        else:
            assert abs(exact - int(v)) <= exact * 2e-15


def test_binary_search_matches_reference(oracle, prim, bases):
    b = np.array(bases["8_22_0"]["words"], dtype=np.uint64)
    q = prim["bsearch"][:, 0]
    got = oracle.find_indices(b, q)
    assert np.array_equal(got, prim["bsearch"][:, 1])
    assert (got == oracle.MISS).sum() >= 500


@pytest.mark.parametrize("key", ["2_8_0", "4_10_0", "4_10_-2", "6_16_0", "6_16_4", "8_22_0", "8_22_2",
                                 "10_28_0", "10_28_2", "10_28_4", "10_28_6", "10_28_8", "11_31_0"])
def test_basis_matches_reference_scan(oracle, bases, key):
    ent = bases[key]
    b = oracle.basis(ent["N"], ent["norb"], ent["two_lz"])
    assert len(b) == ent["dim"]
    assert hashlib.sha256(b.astype("<u8").tobytes()).hexdigest() == ent["sha256"]
    if "words" in ent:
        assert np.array_equal(b, np.array(ent["words"], dtype=np.uint64))


def test_sector_dimensions_of_measured_configs(bases):
    dims = {k: v["dim"] for k, v in bases.items()}
    assert dims["8_22_0"] == 8512
    assert dims["11_31_0"] == 1371535
    assert [dims[f"10_28_{t}"] for t in (0, 2, 4, 6, 8)] == [246448, 246129, 245394, 244037, 242268]
    assert dims["12_34_0"] == 7764392


def test_oracle_against_compiled_reference_random(oracle):
    R = oracle.ref_lib()
    if R is None:
        pytest.skip("reference sources not present here (fixtures above pin the oracle)")
    import ctypes
    rng = np.random.default_rng(7)
    for _ in range(20000):
        norb = int(rng.integers(4, 41))
        N = int(rng.integers(1, min(norb, 16)))
        occ = rng.choice(norb, size=N, replace=False)
        st = sum(1 << int(o) for o in occ)
        ks = [int(x) for x in rng.integers(0, norb, size=4)]
        if rng.random() < 0.6 and N >= 2:
            ks[2], ks[3] = (int(x) for x in rng.choice(occ, size=2, replace=False))
        s = ctypes.c_int(0)
        o = R.ref_evaluate_cdcdcc(ctypes.byref(s), 1 << ks[0], 1 << ks[1], 1 << ks[2], 1 << ks[3], st, 1 << (norb - 1))
        o2, s2 = oracle.evaluate_cdcdcc(*ks, st, norb)
        assert s2 == s.value and (s2 == 0 or o2 == o)
        assert oracle.next_hamming(st) == R.ref_next_hamming(st)


# ------------------------- the reference's own quartic build and observables

@pytest.fixture(scope="module")
def ref_ham():
    with open(os.path.join(GOLD, "ref_hamiltonians.json")) as f:
        return json.load(f)


def _pp(oracle, kind, norb):
    return oracle.odd_coulomb_list(norb) if kind == "coulomb" else np.array([0.0, 1.0])


def test_build_upper_matches_reference_crs(oracle, ref_ham):
    # Add_CdCdCC_Terms (spinless_fermion_hamiltonian.hpp:282-436) with the
    # reference's hash accumulation, trim and CRS conversion: the oracle's
    # upper-triangle CRS has the same rows, columns and FP64 value bits
    for key, ent in ref_ham["crs"].items():
        N, norb, tlz = ent["N"], ent["norb"], ent["two_lz"]
        b = oracle.basis(N, norb, tlz)
        assert len(b) == ent["dim"], key
        kt, vt = oracle.quartic_tables(norb, _pp(oracle, ent["pseudopotentials"], norb))
        rp, col, val = oracle.build_upper(b, norb, kt, vt)
        assert int(rp[-1]) == ent["nnz_upper"], key
        assert oracle.crs_digest(rp, col, val) == ent["sha256"], key


def _seeded(seed, nev, n, complex_=False):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((nev, n))
    if complex_:
        v = v + 1j * rng.standard_normal((nev, n))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def test_observables_match_reference(oracle, ref_ham):
    # DensityFunction, DensityDensityFunction, GetParticipationRatio
    # (fermion_observables.hpp:48-200, 528-562) on seeded unit vectors
    g = ref_ham["observables"]
    N, norb, tlz = g["N"], g["norb"], g["two_lz"]
    b = oracle.basis(N, norb, tlz)
    ev = _seeded(g["seed"], g["nev"], len(b))
    for e, ref in enumerate(g["vectors"]):
        d = oracle.density(b, ev[e], norb)
        assert np.max(np.abs(d - np.array(ref["density"]))) <= 1e-13
        dd = oracle.density_density(b, ev[e], norb)
        assert np.max(np.abs(dd.ravel() - np.array(ref["density_density"]))) <= 1e-13
        pr = oracle.participation_ratio(ev[e])
        assert abs(pr - ref["participation_ratio"]) <= 1e-13 * ref["participation_ratio"]


def test_most_probable_matches_reference_on_complex_vectors(oracle, ref_ham):
    # GetMostProbable (fermion_observables.hpp:437-517) for complex vectors
    # (the reference's routine copies complex-sized blocks, so it ranks real
    # vectors' amplitudes in pairs; the build ranks |psi| as intended)
    g = ref_ham["most_probable"]
    N, norb, tlz, k = g["N"], g["norb"], g["two_lz"], g["k"]
    b = oracle.basis(N, norb, tlz)
    ev = _seeded(g["seed"], g["nev"], len(b), complex_=True)
    states = np.array(g["states"], dtype=np.uint64).reshape(g["nev"], k)
    amps = (np.array(g["amplitudes_re"]) + 1j * np.array(g["amplitudes_im"])).reshape(g["nev"], k)
    for e in range(g["nev"]):
        w, a = oracle.most_probable(b, ev[e], k)
        assert np.array_equal(w, states[e])
        assert np.max(np.abs(a - amps[e])) <= 1e-15


def test_oracle_against_compiled_reference_hamiltonian(oracle):
    R = oracle.ref_ham_lib()
    if R is None:
        pytest.skip("reference sources not present here (the fixtures above pin the oracle)")
    rng = np.random.default_rng(21)
    for (N, norb, tlz) in [(5, 14, 1), (6, 17, 0), (7, 18, 3)]:
        b = oracle.basis(N, norb, tlz)
        assert np.array_equal(oracle.ref_basis(R, N, norb, tlz), b)
        pp = oracle.odd_coulomb_list(norb)
        pp = pp * rng.uniform(0.5, 1.5, len(pp))
        kt, vt = oracle.quartic_tables(norb, pp)
        ref = oracle.ref_build_upper(R, N, norb, tlz, kt, vt)
        got = oracle.build_upper(b, norb, kt, vt)
        assert np.array_equal(ref[0], got[0]) and np.array_equal(ref[1], got[1])
        assert np.array_equal(ref[2].view(np.uint64), got[2].view(np.uint64))


def test_two_level_build_matches_reference_crs(oracle, ref_ham):
    # the two-level model's build (two_level_pseudopotential_model.cpp:190-215)
    for key, ent in ref_ham["crs_two_level"].items():
        N, norb0, tlz = ent["N"], ent["norb0"], ent["two_lz"]
        f, s = oracle.basis2(N, norb0, tlz)
        assert len(f) == ent["dim"], key
        kt0, vt0 = oracle.quartic_tables(norb0, oracle.odd_coulomb_list(norb0))
        kt1, vt1 = oracle.quartic_tables(norb0 + 2, oracle.odd_coulomb_list(norb0 + 2))
        e0 = np.linspace(-0.3, 0.2, norb0) if ent["energies"] else None
        e1 = np.linspace(0.9, 1.4, norb0 + 2) if ent["energies"] else None
        rp, col, val = oracle.build_upper2(f, s, norb0, kt0, vt0, kt1, vt1, e0, e1)
        assert int(rp[-1]) == ent["nnz_upper"], key
        assert oracle.crs_digest(rp, col, val) == ent["sha256"], key


def test_two_level_oracle_against_compiled_reference(oracle):
    R = oracle.ref_ham_lib()
    if R is None:
        pytest.skip("reference sources not present here (the fixtures above pin the oracle)")
    rng = np.random.default_rng(5)
    for (N, norb0, tlz) in [(3, 5, 0), (5, 7, 2), (5, 9, 2)]:
        f, s = oracle.basis2(N, norb0, tlz)
        rf, rs = oracle.ref_basis2(R, N, norb0, tlz)
        assert np.array_equal(f, rf) and np.array_equal(s, rs)
        p0 = oracle.odd_coulomb_list(norb0) * rng.uniform(0.5, 1.5, norb0 - 1)
        p1 = oracle.odd_coulomb_list(norb0 + 2) * rng.uniform(0.5, 1.5, norb0 + 1)
        kt0, vt0 = oracle.quartic_tables(norb0, p0)
        kt1, vt1 = oracle.quartic_tables(norb0 + 2, p1)
        e0, e1 = rng.uniform(-1, 1, norb0), rng.uniform(0, 2, norb0 + 2)
        ref = oracle.ref_build_upper2(R, N, norb0, tlz, kt0, vt0, kt1, vt1, e0, e1)
        got = oracle.build_upper2(f, s, norb0, kt0, vt0, kt1, vt1, e0, e1)
        assert np.array_equal(ref[0], got[0]) and np.array_equal(ref[1], got[1])
        assert np.array_equal(ref[2].view(np.uint64), got[2].view(np.uint64))


def _ofl_case(oracle, ent):
    N, X, Y = ent["N"], ent["X"], ent["Y"]
    K = X * Y
    kt, vt = oracle.ofl_tables(X, Y, K + N)
    e = (np.linspace(-0.4, 0.6, K) + 1e-3j * np.arange(K)) if ent["energies"] else None
    return kt, vt, e


def test_complex_build_matches_reference_crs(oracle, ref_ham):
    # the optical-flux-lattice model's complex build (interacting_ofl_model.cpp:
    # 1034-1052) on seeded array-format tables; the Python loops and their C
    # port both give the reference's CRS
    for key, ent in ref_ham["crs_complex"].items():
        N, X, Y, kx, ky = ent["N"], ent["X"], ent["Y"], ent["kx"], ent["ky"]
        b = oracle.basis_momentum(N, X, Y, kx, ky)
        assert len(b) == ent["dim"], key
        kt, vt, e = _ofl_case(oracle, ent)
        rp, col, val = oracle.build_upper_complex_c(b, X * Y, kt, vt, e)
        assert int(rp[-1]) == ent["nnz_upper"], key
        assert oracle.crs_digest(rp, col, val.view(np.float64)) == ent["sha256"], key
        if ent["dim"] < 500:
            rp2, col2, val2 = oracle.build_upper_complex(b, X * Y, kt, vt, e)
            assert oracle.crs_digest(rp2, col2, np.asarray(val2).view(np.float64)) == ent["sha256"], key


def test_complex_oracle_against_compiled_reference(oracle):
    R = oracle.ref_ofl_lib()
    if R is None:
        pytest.skip("reference sources not present here (the fixtures above pin the oracle)")
    for (N, X, Y, kx, ky) in [(4, 2, 5, 1, 3), (5, 3, 5, 2, 0)]:
        b = oracle.basis_momentum(N, X, Y, kx, ky)
        assert np.array_equal(oracle.ref_basis_momentum(R, N, X, Y, kx, ky), b)
        kt, vt = oracle.ofl_tables(X, Y, 7 * N + X)
        e = np.linspace(-1.0, 1.0, X * Y) + 0.01j
        ref = oracle.ref_build_upper_complex(R, N, X, Y, kx, ky, kt, vt, e)
        got = oracle.build_upper_complex_c(b, X * Y, kt, vt, e)
        assert np.array_equal(ref[0], got[0]) and np.array_equal(ref[1], got[1])
        assert np.array_equal(ref[2].view(np.uint64), got[2].view(np.uint64))
