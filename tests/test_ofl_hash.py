"""Hash-table term format of the optical-flux-lattice model (host side): the
tables filled from the array format, their files in the reference's binary
and text layouts, and files the reference itself wrote
(tests/golden/ofl_hash_ref_2x3_*, tests/golden/make_golden_ham.py).  The
builds from hash tables are in tests/test_gpu_ofl.py."""
import json
import os

import numpy as np
import pytest

import hamiltonian_diagonalization_gb300 as ed

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def array_and_hash(oracle, X, Y, seed):
    kt, vt = oracle.ofl_tables(X, Y, seed)
    T = ed.ComplexQuarticTermTables(X, Y, kt, vt)
    H = ed.QuarticTermHashTables()
    H.Initialize(X * Y)
    H.SetQuarticFromArray(T)
    return T, H


def test_keys_pack_as_the_reference():
    assert ed.hash_key(3, 7) == (3 << 32) | 7
    assert ed.hash_key(1, 2, 3) == (1 << 48) | (2 << 32) | (3 << 16)
    assert ed.hash_key(1, 2, 3, 4) == (1 << 48) | (2 << 32) | (3 << 16) | 4


@pytest.mark.parametrize("grid", [(2, 3), (3, 4), (4, 5)])
def test_hash_tables_answer_as_the_arrays(oracle, grid):
    X, Y = grid
    K = X * Y
    T, H = array_and_hash(oracle, X, Y, 7)
    assert len(H.kkeys) == K ** 3 and len(H.vkeys) == K ** 3 and H.GetMaxKCount() == 1
    rng = np.random.default_rng(K)
    for k2, k3, k4 in rng.integers(0, K, (300, 3)):
        k1 = T.GetK1(k2, k3, k4)[0]
        assert H.GetK1(k2, k3, k4) == [k1]
        assert H.GetVkkkk(k1, k2, k3, k4) == T.GetVkkkk(k1, k2, k3, k4)
    # absent terms read as zero
    k1 = (T.GetK1(0, 1, 2)[0] + 1) % K
    assert H.GetVkkkk(k1, 0, 1, 2) == 0


@pytest.mark.parametrize("fmt", ["binary", "text"])
def test_file_round_trip(oracle, tmp_path, fmt):
    _, H = array_and_hash(oracle, 3, 4, 9)
    D = ed.QuadraticTermHashTables()
    D.SetQuadraticFromArray(np.linspace(-0.4, 0.6, 12) + 1e-3j * np.arange(12))
    for tab, cls in ((H, ed.QuarticTermHashTables), (D, ed.QuadraticTermHashTables)):
        path = str(tmp_path / f"t.{fmt}")
        tab.ToFile(path, fmt)
        back = cls()
        back.FromFile(path, fmt)
        assert np.array_equal(back.kkeys, tab.kkeys) and np.array_equal(back.kvals, tab.kvals)
        assert np.array_equal(back.vkeys, tab.vkeys)
        if fmt == "binary":
            assert np.array_equal(back.vvals, tab.vvals)
        else:   # 15 significant digits, as the reference writes text
            assert np.max(np.abs(back.vvals - tab.vvals)) <= 1e-14 * max(1.0, np.abs(tab.vvals).max())
    if fmt == "text":
        lines = open(str(tmp_path / "t.text")).read().splitlines()
        assert lines[0] == "# File contains term table data in hash table format"
        assert lines[1:3] == ["12", "1"] and lines[3] == "0\t0"


def test_wrong_header_refused(tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("# File contains term table data in array format\n0\n3\n0\n4\n")
    with pytest.raises(ed.EDError):
        ed.QuarticTermHashTables().FromFile(str(p), "text")


@pytest.mark.parametrize("ext,fmt", [("bin", "binary"), ("txt", "text")])
def test_reads_reference_written_files(oracle, ext, fmt):
    # files the reference wrote from oracle.ofl_tables(2, 3, 11): every entry
    # is ours; the reference's writer drops exactly one entry of each table,
    # the second-smallest key (its gather's duplicate removal skips it)
    _, H = array_and_hash(oracle, 2, 3, 11)
    D = ed.QuadraticTermHashTables()
    D.SetQuadraticFromArray(np.linspace(-0.4, 0.6, 6) + 1e-3j * np.arange(6))
    for name, ours, cls in (("quartic", H, ed.QuarticTermHashTables), ("quadratic", D, ed.QuadraticTermHashTables)):
        ref = cls()
        ref.FromFile(os.path.join(GOLDEN, f"ofl_hash_ref_2x3_{name}.{ext}"), fmt)
        tol = 0.0 if fmt == "binary" else 1e-14
        kd = dict(zip(ours.kkeys.tolist(), ours.kvals.tolist()))
        vd = dict(zip(ours.vkeys.tolist(), ours.vvals.tolist()))
        for k, v in zip(ref.kkeys.tolist(), ref.kvals.tolist()):
            assert kd[k] == v
        for k, v in zip(ref.vkeys.tolist(), ref.vvals.tolist()):
            assert abs(vd[k] - v) <= tol * max(1.0, abs(v))
        for keys, mine in ((ref.kkeys, ours.kkeys), (ref.vkeys, ours.vkeys)):
            missing = sorted(set(mine.tolist()) - set(keys.tolist()))
            assert missing == [sorted(mine.tolist())[1]], (name, missing)


def test_reference_writer_defect_recorded():
    gold = json.load(open(os.path.join(GOLDEN, "ref_hamiltonians.json")))
    for key, d in gold["hash_writer_defect"].items():
        assert d["written_k"] == d["expected"] - 1 and d["written_v"] == d["expected"] - 1, key
        assert len(d["missing_k_keys"]) == 1 and len(d["missing_v_keys"]) == 1, key


def test_model_converts_and_stores_under_the_reference_names(oracle, tmp_path):
    kt, vt = oracle.ofl_tables(3, 4, 5)
    m = ed.InteractingOflModel(4, 3, 4, ed.ComplexQuarticTermTables(3, 4, kt, vt), np.linspace(0, 1, 12))
    with pytest.raises(ed.EDError):
        m.TermsToFile(str(tmp_path))
    m.ConvertTableFormat()
    assert m.m_tableFormat == "hash" and m.tables is None
    m.TermsToFile(str(tmp_path), "text")
    names = sorted(os.listdir(str(tmp_path)))
    assert names == ["quadratic_coefficient_table_kx_3_ky_4.dat", "quartic_coefficient_table_kx_3_ky_4.dat"]
    m2 = ed.InteractingOflModel(4, 3, 4, None)
    m2.TermsFromFile(str(tmp_path), "text")
    assert m2.m_tableFormat == "hash" and len(m2.m_quarticHashTables.kkeys) == 12 ** 3
