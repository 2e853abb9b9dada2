"""Host-side term tables of the library (C++) against the exact oracle:
Clebsch-Gordan coefficients, the Coulomb pseudopotentials, the k/V tables
(pseudopotential_model_base.hpp:62-229) and the derived per-hop table."""
import numpy as np
import pytest

import hamiltonian_diagonalization_gb300 as ed


def test_clebsch_gordan_vs_exact_racah(edlib, oracle):
    rng = np.random.default_rng(3)
    worst = 0.0
    for _ in range(4000):
        tj1, tj2 = (int(x) for x in rng.integers(0, 61, size=2))
        tJ = int(rng.choice(np.arange(abs(tj1 - tj2), tj1 + tj2 + 1, 2)))
        tm1 = int(rng.choice(np.arange(-tj1, tj1 + 1, 2)))
        tm2 = int(rng.choice(np.arange(-tj2, tj2 + 1, 2)))
        tM = tm1 + tm2
        if abs(tM) > tJ:
            continue
        a = ed.clebsch_gordan(tj1, tm1, tj2, tm2, tJ, tM)
        b = oracle.cg_exact(tj1, tm1, tj2, tm2, tJ, tM)
        if b == 0.0:
            assert a == 0.0
        else:
            worst = max(worst, abs(a - b) / abs(b))
    assert worst < 2e-15


def test_clebsch_gordan_range_limit(edlib):
    # j1 + j2 + J beyond 120 is outside the exact-integer range: reported as 0
    assert ed.clebsch_gordan(80, 0, 80, 0, 160, 0) == 0.0
    assert ed.clebsch_gordan(60, 0, 60, 0, 120, 0) != 0.0


def test_clebsch_gordan_selection_rules(edlib):
    assert ed.clebsch_gordan(2, 2, 2, 0, 4, 0) == 0.0      # M != m1 + m2
    assert ed.clebsch_gordan(2, 2, 2, 2, 2, 4) == 0.0      # |M| > J
    assert ed.clebsch_gordan(1, 1, 1, 1, 4, 2) == 0.0      # triangle
    assert abs(ed.clebsch_gordan(1, 1, 1, -1, 0, 0) - np.sqrt(0.5)) < 1e-16
    assert abs(ed.clebsch_gordan(1, -1, 1, 1, 0, 0) + np.sqrt(0.5)) < 1e-16


def test_coulomb_pseudopotentials_exact(edlib, oracle):
    for norb in (4, 8, 22, 28, 31, 34, 40):
        a = ed.coulomb_pseudopotentials(norb)
        b = oracle.coulomb_pseudopotentials(norb)
        assert np.max(np.abs(a - b) / np.abs(b)) < 1e-15


@pytest.mark.parametrize("norb", [4, 8, 13, 22, 28])
def test_quartic_tables_vs_oracle(edlib, oracle, norb):
    rng = np.random.default_rng(norb)
    for pp in (oracle.odd_coulomb_list(norb), rng.uniform(-1, 2, size=norb - 1), [0.0, 1.0]):
        T = ed.QuarticTermTables(norb, pp)
        kt, vt = oracle.quartic_tables(norb, pp)
        assert np.array_equal(T.m_kTable, kt)
        assert np.max(np.abs(T.m_vTable - vt)) <= 1e-13 * max(1.0, np.max(np.abs(vt)))


def test_too_many_pseudopotentials_rejected(edlib):
    with pytest.raises(ed.EDError) as e:
        ed.QuarticTermTables(8, np.ones(8))
    assert e.value.status == 1


def test_momentum_table_checked(edlib, oracle):
    kt, vt = oracle.quartic_tables(6, [0.0, 1.0])
    kt = kt.copy()
    kt[5] = (int(kt[5]) + 1) % 6
    T = ed.QuarticTermTables(6, ktable=kt, vtable=vt)
    with pytest.raises(ed.EDError):
        T.handle()          # device upload checks the table first (host-side check)


def test_reference_table_accessors(edlib):
    T = ed.QuarticTermTables(8, [0.0, 1.0])
    K = 8
    for k4 in range(K):
        for k3 in range(K):
            for k2 in range(K):
                k1 = k3 + k4 - k2
                got = T.GetK1(k2, k3, k4)
                assert got == ([k1] if 0 <= k1 < K else [])
    assert T.GetMaxKCount() == 1
