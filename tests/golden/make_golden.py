"""Generate the golden fixtures of tests/golden/ from the reference's OWN code.

The reference repository ships no tests or fixtures for this path, so the
fixtures here are outputs of the reference's primitives, compiled from its
sources by ``make -C oracle ref REFSRC=<its src directory>`` into
oracle/_ref/libref.so (a shim of ours calls them through a C ABI).  Run in a
container where the reference tree is present (REFSRC names its src
directory; the default is where this build mounts it):

    REFSRC=/root/reference/src python tests/golden/make_golden.py

Outputs (committed, a few hundred KB):
  ref_primitives.npz  random inputs and the reference's outputs for
                      Evaluate_CdCdCC, NextHammingNumber64,
                      GenerateHammingNumber, HammingWeight64Iterative,
                      Base2Log, TestAngularMomentumSector, BinarySearch,
                      BinomialFromTable
  ref_bases.json      sector dimensions and SHA-256 digests of the basis words
                      (little-endian uint64, ascending) produced by the
                      reference's own scan for every measured configuration,
                      plus the full word list of the smallest ones
"""
import ctypes
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

SEED = 20261203


def main():
    O.build_ref(os.environ.get("REFSRC") or "/root/reference/src")
    R = O.ref_lib()
    if R is None:
        raise SystemExit("reference sources not present: cannot build oracle/_ref")
    R.ref_basis_scan.restype = ctypes.c_uint64
    R.ref_basis_scan.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64)]
    rng = np.random.default_rng(SEED)
    out = {}

    # Evaluate_CdCdCC on random states: half with operators drawn from the
    # state's own occupation (mostly non-vanishing), half uniform.
    M = 20000
    norbs = rng.choice([8, 22, 28, 31, 34], size=M)
    rec = np.zeros((M, 8), dtype=np.uint64)  # norb k1 k2 k3 k4 state out sign(+2 offset)
    for t in range(M):
        norb = int(norbs[t])
        N = int(rng.integers(2, min(norb, 13)))
        occ = rng.choice(norb, size=N, replace=False)
        state = 0
        for o in occ:
            state |= 1 << int(o)
        if t % 2 == 0:
            k3, k4 = (int(x) for x in rng.choice(occ, size=2, replace=False))
            k1, k2 = (int(x) for x in rng.integers(0, norb, size=2))
        else:
            k1, k2, k3, k4 = (int(x) for x in rng.integers(0, norb, size=4))
        s = ctypes.c_int(0)
        o = R.ref_evaluate_cdcdcc(ctypes.byref(s), 1 << k1, 1 << k2, 1 << k3, 1 << k4, state, 1 << (norb - 1))
        rec[t] = [norb, k1, k2, k3, k4, state, o, s.value + 2]
    out["cdcdcc"] = rec

    # NextHammingNumber64 chains and GenerateHammingNumber at random indices
    nh = np.zeros((4000, 2), dtype=np.uint64)
    for t in range(4000):
        w = int(rng.integers(1, 20))
        x = int(rng.integers(1, 1 << 40))
        # force popcount w by taking the lowest w set bits of a random mask
        bits = [b for b in range(64) if (x >> b) & 1][:w]
        x = sum(1 << b for b in bits) if bits else 1
        nh[t] = [x, R.ref_next_hamming(x)]
    out["next_hamming"] = nh
    gh = np.zeros((4000, 3), dtype=np.uint64)
    for t in range(4000):
        norb = int(rng.integers(4, 35))
        w = int(rng.integers(1, min(norb, 13)))
        full = O.binomial(norb, w)
        idx = int(rng.integers(0, full))
        gh[t] = [w, idx, R.ref_generate_hamming(w, idx)]
    out["generate_hamming"] = gh

    hw = rng.integers(0, 1 << 62, size=2000, dtype=np.int64).astype(np.uint64)
    out["hamming_weight"] = np.stack([hw, np.array([R.ref_hamming_weight(int(x)) for x in hw], dtype=np.uint64)], 1)
    b2 = np.array([1 << int(p) for p in rng.integers(0, 64, size=500)], dtype=np.uint64)
    out["base2log"] = np.stack([b2, np.array([R.ref_base2log(int(x)) for x in b2], dtype=np.uint64)], 1)

    lz = np.zeros((4000, 4), dtype=np.int64)
    for t in range(4000):
        norb = int(rng.integers(4, 35))
        N = int(rng.integers(1, min(norb, 13)))
        occ = rng.choice(norb, size=N, replace=False)
        state = sum(1 << int(o) for o in occ)
        tlz = int(sum(2 * int(o) - (norb - 1) for o in occ))
        if t % 3 == 1:
            tlz += 2
        lz[t] = [state, tlz, norb - 1, R.ref_lz_ok(state, tlz, norb - 1)]
    out["lz_ok"] = lz

    binom = np.array([[n, k, R.ref_binomial(n, k)] for n in range(0, 65) for k in range(0, n + 1)], dtype=np.int64)
    out["binomial"] = binom

    # BinarySearch hits and misses on the config-0 basis
    n_b = int(R.ref_basis_scan(8, 22, 0, None))
    b = np.empty(n_b, dtype=np.uint64)
    R.ref_basis_scan(8, 22, 0, b.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    q = np.concatenate([b[rng.integers(0, n_b, 2000)], O.basis(8, 22, 2)[:500],
                        np.array([0, 1, int(b[0]) - 1, int(b[-1]) + 1], dtype=np.uint64)])
    bp = b.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    out["bsearch"] = np.stack([q, np.array([R.ref_binary_search(int(x), bp, n_b) for x in q], dtype=np.uint64)], 1)
    np.savez_compressed(os.path.join(HERE, "ref_primitives.npz"), **out)

    bases = {}
    cfgs = [(8, 22, 0), (8, 22, 2), (4, 10, 0), (4, 10, -2), (2, 8, 0), (6, 16, 0), (6, 16, 4),
            (10, 28, 0), (10, 28, 2), (10, 28, 4), (10, 28, 6), (10, 28, 8),
            (11, 31, 0), (12, 34, 0)]
    for (N, norb, tlz) in cfgs:
        n = int(R.ref_basis_scan(N, norb, tlz, None))
        words = np.empty(n, dtype=np.uint64)
        if n:
            R.ref_basis_scan(N, norb, tlz, words.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
        ent = {"N": N, "norb": norb, "two_lz": tlz, "dim": n,
               "sha256": hashlib.sha256(words.astype("<u8").tobytes()).hexdigest()}
        if n <= 10000:
            ent["words"] = [int(x) for x in words]
        bases[f"{N}_{norb}_{tlz}"] = ent
        print(N, norb, tlz, n, flush=True)
    with open(os.path.join(HERE, "ref_bases.json"), "w") as f:
        json.dump(bases, f)


if __name__ == "__main__":
    main()
