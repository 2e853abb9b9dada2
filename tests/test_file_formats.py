"""The reference's file formats (eigensystem, CRS, quartic term tables): the
layouts written by hamiltonian_base.hpp:1204-1304, crs_sparse_matrix.hpp:662-740
and term_tables_base.hpp:179-335, and round trips through the engine's
readers.  Host-only except the CRS files, which start from a device matrix."""
import struct

import numpy as np
import pytest

import hamiltonian_diagonalization_gb300 as ed
from hamiltonian_diagonalization_gb300.host import eigensystem_from_file, eigensystem_to_file


def test_eigensystem_text_layout_and_round_trip(tmp_path):
    ev = np.array([-1.2345678901234567, 0.5, 3.0e-7])
    vec = np.random.default_rng(0).standard_normal((3, 5))
    p = tmp_path / "eig.dat"
    eigensystem_to_file(str(p), ev, vec, "text")
    lines = p.read_text().splitlines()
    assert lines[:2] == ["##  NBR EIGENVALUES", "3"]
    assert lines[2] == "##  EIGENVALUES"
    # std::setprecision(15), default float notation: %.15g
    assert lines[3:6] == ["%.15g" % x for x in ev]
    assert lines[6:8] == ["##  FOCK SPACE DIMENSION", "5"]
    assert lines[8] == "##  EIGENVECTORS"
    assert lines[9:] == ["%.15g" % x for x in vec.ravel()]
    ev2, vec2 = eigensystem_from_file(str(p), "text")
    assert np.allclose(ev2, ev, rtol=1e-14, atol=0) and np.allclose(vec2, vec, rtol=1e-14, atol=0)


def test_eigensystem_values_only_and_binary(tmp_path):
    ev = np.array([1.0, 2.0])
    p = tmp_path / "vals.dat"
    eigensystem_to_file(str(p), ev, None, "text")
    assert p.read_text() == "##  NBR EIGENVALUES\n2\n##  EIGENVALUES\n1\n2\n"
    ev2, vec2 = eigensystem_from_file(str(p), "text")
    assert np.array_equal(ev2, ev) and vec2 is None
    vec = np.random.default_rng(1).standard_normal((2, 7))
    b = tmp_path / "eig.bin"
    eigensystem_to_file(str(b), ev, vec, "binary")
    raw = b.read_bytes()
    assert struct.unpack("<I", raw[:4])[0] == 2
    assert np.array_equal(np.frombuffer(raw[4:20], dtype=np.float64), ev)
    assert struct.unpack("<I", raw[20:24])[0] == 7
    assert np.array_equal(np.frombuffer(raw[24:], dtype=np.float64), vec.ravel())
    ev3, vec3 = eigensystem_from_file(str(b), "binary")
    assert np.array_equal(ev3, ev) and np.array_equal(vec3, vec)


@pytest.mark.parametrize("fmt", ["text", "binary"])
def test_quartic_tables_round_trip(tmp_path, fmt):
    norb = 9
    t = ed.QuarticTermTables(norb, ed.odd_coulomb_list(norb))
    p = tmp_path / ("tables." + fmt)
    t.ToFile(str(p), fmt)
    t2 = ed.QuarticTermTables.FromFile(str(p), fmt)
    assert t2.m_kMax == norb
    assert np.array_equal(t2.m_kTable, t.m_kTable)
    if fmt == "binary":
        assert np.array_equal(t2.m_vTable, t.m_vTable)
        raw = p.read_bytes()
        hlen = struct.unpack("<I", raw[:4])[0]
        assert raw[4:4 + hlen] == b"# File contains term table data in array format"
        assert struct.unpack("<II", raw[4 + hlen:12 + hlen]) == (4, norb)
        assert len(raw) == 12 + hlen + norb ** 3 * (2 + 8)
    else:
        assert np.allclose(t2.m_vTable, t.m_vTable, rtol=1e-14, atol=0)
        lines = p.read_text().splitlines()
        assert lines[:3] == ["# File contains term table data in array format", "4", str(norb)]
        k1, k2, k3, k4, v = lines[3 + 1].split("\t")      # (k4, k3, k2) = (0, 0, 1)
        assert (int(k2), int(k3), int(k4)) == (1, 0, 0)
        assert int(k1) == int(t.m_kTable[1]) and v == "%.15g" % t.m_vTable[1]
        assert len(lines) == 3 + norb ** 3


def test_bad_files_are_rejected(tmp_path):
    p = tmp_path / "bad.dat"
    p.write_text("# not a term table\n4\n3\n")
    with pytest.raises(ed.EDError):
        ed.QuarticTermTables.FromFile(str(p), "text")
    with pytest.raises(ed.EDError):
        eigensystem_from_file(str(tmp_path / "missing.dat"), "text")


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", ["text", "binary"])
def test_crs_file_round_trip(cuda, tmp_path, fmt):
    H = ed.SpinlessFermionHamiltonian()
    H.Initialize(6, 16, twoLz=0)
    H.Add_CdCdCC_Terms(ed.QuarticTermTables(16, ed.odd_coulomb_list(16)), store_upper=True)
    A = H.m_crsSparseMatrix
    p = tmp_path / ("h." + fmt)
    A.ToFile(str(p), fmt)
    B = ed.CrsSparseMatrix.FromFile(str(p), fmt, upper=True)
    rp, col, val = A.to_host()
    rp2, col2, val2 = B.to_host()
    assert np.array_equal(rp, rp2) and np.array_equal(col, col2)     # last row kept
    if fmt == "binary":
        assert np.array_equal(val, val2)
    else:
        assert np.allclose(val, val2, rtol=1e-14, atol=0)
        lines = p.read_text().splitlines()
        assert int(lines[0]) == len(col) and int(lines[1]) == len(rp) - 1
        assert len(lines) == 2 + (len(rp) - 1) + len(col)
