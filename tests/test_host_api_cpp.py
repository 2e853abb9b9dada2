"""The reference-shaped C++ host classes (include/ed_host.hpp) compile against
the C ABI here, and drive a whole sector solve on the GPU."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "hamiltonian_diagonalization_gb300")


def compile_demo(tmp_path):
    exe = str(tmp_path / "host_api_demo")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "host_api_demo.cpp"), "-L", PKG, "-ledgb300",
                           f"-Wl,-rpath,{PKG}", "-o", exe])
    return exe


def test_host_classes_compile(edlib, tmp_path):
    assert os.path.exists(compile_demo(tmp_path))


@pytest.mark.gpu
def test_host_classes_solve_sector(cuda, oracle, tmp_path):
    exe = compile_demo(tmp_path)
    out = subprocess.run([exe, "6", "16", "0"], capture_output=True, text=True, timeout=300, cwd=str(tmp_path))
    assert out.returncode == 0, out.stdout + out.stderr
    r = json.loads(out.stdout.strip().splitlines()[-1])
    assert r["ok"] and r["ok_host_product"] and r["rank_ok"]
    # hash-format terms through files: same matrix, same eigenvalues as the arrays
    h = r["ofl_hash"]
    assert h["ok"] and h["lookups_ok"] and h["same_as_array"]
    import scipy.sparse as sp
    pp = oracle.odd_coulomb_list(16)
    b = oracle.basis(6, 16, 0)
    kt, vt = oracle.quartic_tables(16, pp)
    fr, fc, fv = oracle.upper_to_full(*oracle.build_upper(b, 16, kt, vt), len(b))
    ref = np.linalg.eigvalsh(sp.csr_matrix((fv, fc, fr), shape=(len(b), len(b))).toarray())[:3]
    assert r["dim"] == len(b) and r["nnz"] == len(fv)
    assert np.max(np.abs(np.array(r["eigenvalues"]) - ref) / np.abs(ref)) < 1e-10
    assert np.max(np.abs(np.array(r["eigenvalues_host_product"]) - ref) / np.abs(ref)) < 1e-10
    # the ground state's observables through the C++ Observables class
    rho = np.array(r["density"])
    assert abs(r["density_sum"] - 6) < 1e-9 and np.allclose(rho, rho[::-1], atol=1e-8)   # N; Lz reflection
    assert abs(r["dd00"] - rho[0]) < 1e-12 and 1.0 <= r["participation"] <= len(b)
    assert int(r["top_state"]) in set(int(w) for w in b)
    # the two-level sector through TwoLevelSpinlessFermionHamiltonian (every degenerate copy)
    t = r["two_level"]
    assert t["ok"] and t["rank_ok"]
    f, s = oracle.basis2(4, 6, 0)
    kt0, vt0 = oracle.quartic_tables(6, oracle.odd_coulomb_list(6))
    kt1, vt1 = oracle.quartic_tables(8, oracle.odd_coulomb_list(8))
    u = oracle.build_upper2(f, s, 6, kt0, vt0, kt1, vt1, None, np.full(8, 0.4))
    fr, fc, fv = oracle.upper_to_full(*u, len(f))
    ref2 = np.linalg.eigvalsh(sp.csr_matrix((fv, fc, fr), shape=(len(f), len(f))).toarray())[:4]
    assert t["dim"] == len(f) and t["nnz"] == len(fv)
    assert np.max(np.abs(np.array(t["eigenvalues"]) - ref2)) < 1e-10 * max(1.0, np.abs(ref2).max())
    # the complex momentum sector through SpinlessFermionHamiltonian<std::complex<double>>
    c = r["ofl"]
    assert c["ok"]
    X, Y = 3, 4
    K = X * Y
    kt, _ = oracle.ofl_tables(X, Y, 0)
    i = np.arange(len(kt))
    k2 = i % K
    t1 = np.empty(len(kt), dtype=np.int64)
    t2 = np.empty(len(kt), dtype=np.int64)
    for a in range(K):
        for bb in range(a, K):
            base = oracle.ofl_index(a, bb, K) * K
            t1[base:base + K], t2[base:base + K] = a, bb
    re = ((i * 7919) % 1000) / 500.0 - 1.0
    im = np.where((k2 == t1) | (k2 == t2), 0.0, ((i * 104729) % 1000) / 500.0 - 1.0)
    vt = re + 1j * im
    b = oracle.basis_momentum(4, X, Y, 1, 2)
    u = oracle.build_upper_complex(b, K, kt, vt, 0.125 * np.arange(K) + 0j)
    fr, fc, fv = oracle.complex_upper_to_full(*u, len(b))
    ref3 = np.linalg.eigvalsh(sp.csr_matrix((fv, fc, fr), shape=(len(b), len(b))).toarray())[:3]
    assert c["dim"] == len(b) and c["nnz"] == len(fv)
    assert np.max(np.abs(np.array(c["eigenvalues"]) - ref3)) < 1e-10 * max(1.0, np.abs(ref3).max())


@pytest.mark.gpu
def test_reference_model_sequence_runs_as_written(cuda, oracle, tmp_path):
    # the reference's BuildFockBasis -> BuildHamiltonian -> BaseDiagonalize
    # sequence through ed_host.hpp: a std::bind(TestAngularMomentumSector)
    # basis, SetFockBasis, Initialize, Add_CdCdCC_Terms, then FullDiagonalize
    # (dimension < 60) or LanczosDiagonalize(&quadratic, &quartic, mv, nev, mpi)
    import scipy.sparse as sp
    exe = compile_demo(tmp_path)
    out = subprocess.run([exe, "6", "16", "2"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    r = json.loads(out.stdout.strip().splitlines()[-1])
    assert r["all_sectors_refused"]
    seq = r["reference_sequence"]
    assert [c["full"] for c in seq] == [False, True]
    for c in seq:
        assert c["ok"]
        b = oracle.basis(c["N"], c["norb"], c["two_lz"])
        assert c["dim"] == len(b)
        kt, vt = oracle.quartic_tables(c["norb"], oracle.odd_coulomb_list(c["norb"]))
        fr, fc, fv = oracle.upper_to_full(*oracle.build_upper(b, c["norb"], kt, vt), len(b))
        ref = np.linalg.eigvalsh(sp.csr_matrix((fv, fc, fr), shape=(len(b), len(b))).toarray())[:len(c["eigenvalues"])]
        assert np.max(np.abs(np.array(c["eigenvalues"]) - ref)) <= 1e-10 * max(1.0, np.abs(ref).max())
