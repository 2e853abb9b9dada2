"""Generate tests/golden/ref_hamiltonians.json from the reference's OWN sector
basis, quartic Hamiltonian build and observables.

The reference's FermionFockBasis::GenerateFockSpace,
SpinlessFermionHamiltonian<double>::Add_CdCdCC_Terms (mapped storage, trim,
CRS conversion) and Observables are compiled from its sources by
``make -C oracle ref REFSRC=<its src directory>`` into
oracle/_ref/libref_ham.so (oracle/ref_ham_shim.cpp drives them through a C
ABI, against the one-rank MPI and compile-only Boost stand-ins in
oracle/ref_stubs/).  Run where the reference tree is present:

    REFSRC=/root/reference/src python tests/golden/make_golden_ham.py

Outputs (committed):
  ref_hamiltonians.json
    crs          per sector and pseudopotential list: dimension, stored
                 (upper-triangle) elements and the SHA-256 of the reference's
                 CRS (row pointers as int64, columns as int32, values as FP64
                 bits), built from the term tables the oracle computes
    crs_two_level  the same for the two-Landau-level model's build
    crs_complex  the same for the optical-flux-lattice model's complex build
                 (values as (re, im) FP64 bits), on seeded array-format tables
    observables  density, density-density and participation ratio of seeded
                 unit vectors on one sector
    most_probable  the reference's most probable states and amplitudes of
                 seeded complex unit vectors (its routine is only sound for
                 complex vectors)
    crs_complex_hash  the same complex builds through the reference's
                 hash-table path (TermsFromFile + the hash branch of
                 BuildHamiltonian) from hash-table files written by this
                 project's writer (ed_term_hash_write), binary and text
    hash_writer_defect  the entries the reference's own hash-table writer
                 drops (its gather's duplicate removal skips the second-
                 smallest key), for each grid of crs_complex_hash
  ofl_hash_ref_2x3_{quartic,quadratic}.{bin,txt}
                 hash-table files written by the reference itself (2 x 3 grid,
                 tables oracle.ofl_tables(2, 3, 11), energies linspace(-0.4,
                 0.6, 6) + 1e-3 i k), for the reader tests
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

# (N, norb, 2Lz, pseudopotentials): the odd-m LLL Coulomb list, or V1 alone
CRS_CASES = [(6, 16, 2, "coulomb"), (7, 19, 2, "coulomb"), (8, 22, 0, "coulomb"), (8, 22, 6, "coulomb"),
             (9, 24, 1, "coulomb"), (10, 28, 0, "coulomb"), (8, 22, 0, "v1"), (9, 24, 1, "v1")]
# two Landau levels (N, norb0, 2Lz, with occupation energies): odd-m Coulomb
# lists for each level's tables, energies linspace(-0.3, 0.2, norb0) and
# linspace(0.9, 1.4, norb0 + 2)
CRS2_CASES = [(4, 6, 0, True), (5, 8, 1, True), (6, 10, 0, False), (6, 10, 2, True), (7, 12, 1, True)]
# optical flux lattice (N, X, Y, kx, ky, with energies): seeded synthetic
# array-format tables (oracle.ofl_tables, seed X*Y + N), energies
# linspace(-0.4, 0.6, X*Y) + 1e-3 i k
CRSC_CASES = [(3, 3, 4, 1, 2, False), (4, 3, 4, 0, 0, True), (5, 4, 4, 2, 1, True), (6, 4, 5, 0, 3, True),
              (7, 4, 5, 3, 4, True)]
# complex builds through hash-table files (a subset of CRSC_CASES)
CRSCH_CASES = [(3, 3, 4, 1, 2, False), (4, 3, 4, 0, 0, True), (6, 4, 5, 0, 3, True)]
OBS_CASE = (8, 22, 0)
OBS_SEED, OBS_NEV = 11, 2
MP_CASE = (6, 16, 2)
MP_SEED, MP_NEV, MP_K = 12, 2, 12


def pseudopotentials(kind: str, norb: int) -> np.ndarray:
    return O.odd_coulomb_list(norb) if kind == "coulomb" else np.array([0.0, 1.0])


def seeded_vectors(seed: int, nev: int, n: int, complex_: bool = False) -> np.ndarray:
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((nev, n))
    if complex_:
        v = v + 1j * rng.standard_normal((nev, n))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def main():
    O.build_ref(os.environ.get("REFSRC") or "/root/reference/src")
    R = O.ref_ham_lib()
    if R is None:
        raise SystemExit("reference sources not present: cannot build oracle/_ref/libref_ham.so")
    out = {"crs": {}, "observables": {}, "most_probable": {}}
    for (N, norb, tlz, kind) in CRS_CASES:
        kt, vt = O.quartic_tables(norb, pseudopotentials(kind, norb))
        t0 = time.time()
        rp, col, val = O.ref_build_upper(R, N, norb, tlz, kt, vt)
        out["crs"][f"{N}_{norb}_{tlz}_{kind}"] = {"N": N, "norb": norb, "two_lz": tlz, "pseudopotentials": kind,
                                                 "dim": len(rp) - 1, "nnz_upper": int(rp[-1]),
                                                 "sha256": O.crs_digest(rp, col, val)}
        print(N, norb, tlz, kind, len(rp) - 1, int(rp[-1]), f"{time.time() - t0:.1f}s", flush=True)
    out["crs_two_level"] = {}
    for (N, norb0, tlz, en) in CRS2_CASES:
        kt0, vt0 = O.quartic_tables(norb0, O.odd_coulomb_list(norb0))
        kt1, vt1 = O.quartic_tables(norb0 + 2, O.odd_coulomb_list(norb0 + 2))
        e0 = np.linspace(-0.3, 0.2, norb0) if en else None
        e1 = np.linspace(0.9, 1.4, norb0 + 2) if en else None
        t0 = time.time()
        rp, col, val = O.ref_build_upper2(R, N, norb0, tlz, kt0, vt0, kt1, vt1, e0, e1)
        out["crs_two_level"][f"{N}_{norb0}_{tlz}_{int(en)}"] = {
            "N": N, "norb0": norb0, "two_lz": tlz, "energies": en, "dim": len(rp) - 1, "nnz_upper": int(rp[-1]),
            "sha256": O.crs_digest(rp, col, val)}
        print("two-level", N, norb0, tlz, en, len(rp) - 1, int(rp[-1]), f"{time.time() - t0:.1f}s", flush=True)
    Rc = O.ref_ofl_lib()
    out["crs_complex"] = {}
    for (N, X, Y, kx, ky, en) in CRSC_CASES:
        K = X * Y
        kt, vt = O.ofl_tables(X, Y, K + N)
        e = (np.linspace(-0.4, 0.6, K) + 1e-3j * np.arange(K)) if en else None
        t0 = time.time()
        rp, col, val = O.ref_build_upper_complex(Rc, N, X, Y, kx, ky, kt, vt, e)
        out["crs_complex"][f"{N}_{X}_{Y}_{kx}_{ky}_{int(en)}"] = {
            "N": N, "X": X, "Y": Y, "kx": kx, "ky": ky, "energies": en, "dim": len(rp) - 1,
            "nnz_upper": int(rp[-1]), "sha256": O.crs_digest(rp, col, val.view(np.float64))}
        print("complex", N, X, Y, kx, ky, en, len(rp) - 1, int(rp[-1]), f"{time.time() - t0:.1f}s", flush=True)
    out["crs_complex_hash"] = {}
    out["hash_writer_defect"] = {}
    import tempfile
    sys.path.insert(0, ROOT)
    import hamiltonian_diagonalization_gb300 as ed
    tmp = tempfile.mkdtemp()
    for (N, X, Y, kx, ky, en) in CRSCH_CASES:
        K = X * Y
        kt, vt = O.ofl_tables(X, Y, K + N)
        e = (np.linspace(-0.4, 0.6, K) + 1e-3j * np.arange(K)) if en else None
        model = ed.InteractingOflModel(N, X, Y, ed.ComplexQuarticTermTables(X, Y, kt, vt), e)
        model.ConvertTableFormat()
        for fmt in ("binary", "text"):
            d = os.path.join(tmp, f"{N}_{X}_{Y}_{fmt}")
            os.makedirs(d, exist_ok=True)
            model.TermsToFile(d, fmt)
            fq, f4 = model._term_file_names(d)
            rp, col, val = O.ref_build_upper_complex_hash(Rc, N, X, Y, kx, ky, f4, fq, fmt == "binary")
            out["crs_complex_hash"][f"{N}_{X}_{Y}_{kx}_{ky}_{int(en)}_{fmt}"] = {
                "N": N, "X": X, "Y": Y, "kx": kx, "ky": ky, "energies": en, "format": fmt, "dim": len(rp) - 1,
                "nnz_upper": int(rp[-1]), "sha256": O.crs_digest(rp, col, val.view(np.float64))}
            print("complex hash", N, X, Y, kx, ky, en, fmt, len(rp) - 1, int(rp[-1]), flush=True)
        # what the reference's own writer leaves out
        f4, fq = os.path.join(tmp, "ref_q.bin"), os.path.join(tmp, "ref_d.bin")
        O.ref_hash_files(Rc, X, Y, kt, vt, e, f4, fq, True)
        for name, path, full in (("quartic", f4, model.m_quarticHashTables),
                                 ("quadratic", fq, model.m_quadraticHashTables)):
            cls = ed.QuarticTermHashTables if name == "quartic" else ed.QuadraticTermHashTables
            h = cls()
            h.FromFile(path, "binary")
            out["hash_writer_defect"][f"{X}_{Y}_{name}"] = {
                "written_k": len(h.kkeys), "written_v": len(h.vkeys), "expected": len(full.kkeys),
                "missing_k_keys": sorted(set(full.kkeys.tolist()) - set(h.kkeys.tolist())),
                "missing_v_keys": sorted(set(full.vkeys.tolist()) - set(h.vkeys.tolist()))}
    # small reference-written files for the reader tests
    X, Y = 2, 3
    kt, vt = O.ofl_tables(X, Y, 11)
    e = np.linspace(-0.4, 0.6, X * Y) + 1e-3j * np.arange(X * Y)
    for binary, ext in ((True, "bin"), (False, "txt")):
        O.ref_hash_files(Rc, X, Y, kt, vt, e, os.path.join(HERE, f"ofl_hash_ref_2x3_quartic.{ext}"),
                         os.path.join(HERE, f"ofl_hash_ref_2x3_quadratic.{ext}"), binary)
    import ctypes
    f64p = ctypes.POINTER(ctypes.c_double)
    N, norb, tlz = OBS_CASE
    n = len(O.ref_basis(R, N, norb, tlz))
    ev = np.ascontiguousarray(seeded_vectors(OBS_SEED, OBS_NEV, n))
    obs = []
    for e in range(OBS_NEV):
        dens, dd, pr = np.empty(norb), np.empty(norb * norb), np.empty(1)
        R.refh_observables(N, norb, tlz, ev.ctypes.data_as(f64p), OBS_NEV, e, dens.ctypes.data_as(f64p),
                           dd.ctypes.data_as(f64p), pr.ctypes.data_as(f64p))
        obs.append({"density": dens.tolist(), "density_density": dd.tolist(), "participation_ratio": float(pr[0])})
    out["observables"] = {"N": N, "norb": norb, "two_lz": tlz, "seed": OBS_SEED, "nev": OBS_NEV, "vectors": obs}
    N, norb, tlz = MP_CASE
    n = len(O.ref_basis(R, N, norb, tlz))
    evc = seeded_vectors(MP_SEED, MP_NEV, n, complex_=True)
    buf = np.ascontiguousarray(np.stack([evc.real, evc.imag], axis=-1).reshape(-1))
    states = np.empty(MP_K * MP_NEV, dtype=np.uint64)
    amps = np.empty(2 * MP_K * MP_NEV)
    R.refh_most_probable_complex(N, norb, tlz, buf.ctypes.data_as(f64p), MP_NEV, MP_K,
                                 states.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), amps.ctypes.data_as(f64p))
    out["most_probable"] = {"N": N, "norb": norb, "two_lz": tlz, "seed": MP_SEED, "nev": MP_NEV, "k": MP_K,
                            "states": [int(x) for x in states], "amplitudes_re": amps[0::2].tolist(),
                            "amplitudes_im": amps[1::2].tolist()}
    with open(os.path.join(HERE, "ref_hamiltonians.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
