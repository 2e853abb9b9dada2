"""The two-Landau-level oracle (restated TwoLevelFermionFockBasis) pinned by
counting identities: its sectors partition the two-level space of N
particles, dimensions are symmetric under Lz -> -Lz, and the order is the
reference's (first, second) sort.  CPU only."""
from math import comb

import numpy as np
import pytest


@pytest.mark.parametrize("N,norb0", [(2, 3), (3, 5), (4, 6)])
def test_sectors_partition_the_space(oracle, N, norb0):
    norb1 = norb0 + 2
    total = sum(comb(norb0, n0) * comb(norb1, N - n0) for n0 in range(N + 1))
    dims = {}
    span = N * (norb1 - 1)
    for tlz in range(-span, span + 1):
        f, s = oracle.basis2(N, norb0, tlz)
        dims[tlz] = len(f)
        if len(f):
            key = f.astype(object) * (1 << norb1) + s.astype(object)
            assert all(key[i] < key[i + 1] for i in range(len(key) - 1))
            assert all(bin(int(a)).count("1") + bin(int(b)).count("1") == N for a, b in zip(f, s))
    assert sum(dims.values()) == total
    assert all(dims[t] == dims[-t] for t in dims)


@pytest.mark.parametrize("N,norb0,tlz", [(4, 6, 0), (5, 7, 0), (6, 9, 0)])
def test_level_exchange_ladder_commutes_with_h(oracle, N, norb0, tlz):
    """T = L0- L1+ (one level-0 particle an orbital down, one level-1 particle
    an orbital up, coefficients sqrt(i (K0 - i)) and sqrt((K1 - 1 - j)(j + 1)),
    no fermionic sign for a move to a neighbouring orbital) maps the sector to
    itself and commutes with the two-level Hamiltonian: the symmetry the
    device solve uses to generate degenerate copies."""
    import scipy.sparse as sp
    n1 = norb0 + 2
    f, s = oracle.basis2(N, norb0, tlz)
    kt0, vt0 = oracle.quartic_tables(norb0, oracle.odd_coulomb_list(norb0))
    kt1, vt1 = oracle.quartic_tables(n1, np.random.default_rng(norb0).uniform(-1, 2, n1 - 1))
    u = oracle.build_upper2(f, s, norb0, kt0, vt0, kt1, vt1, None, np.full(n1, 0.4))
    fr, fc, fv = oracle.upper_to_full(*u, len(f))
    H = sp.csr_matrix((fv, fc, fr), shape=(len(f), len(f)))
    index = {(int(a), int(b)): i for i, (a, b) in enumerate(zip(f, s))}
    rows, cols, vals = [], [], []
    for r, (a, b) in enumerate(zip(f, s)):
        a, b = int(a), int(b)
        for i in range(1, norb0):
            if not (a >> i) & 1 or (a >> (i - 1)) & 1:
                continue
            for j in range(n1 - 1):
                if not (b >> j) & 1 or (b >> (j + 1)) & 1:
                    continue
                k = index[(a ^ (1 << i) ^ (1 << (i - 1)), b ^ (1 << j) ^ (1 << (j + 1)))]
                rows.append(k)
                cols.append(r)
                vals.append(np.sqrt(i * (norb0 - i)) * np.sqrt((n1 - 1 - j) * (j + 1)))
    T = sp.csr_matrix((vals, (rows, cols)), shape=(len(f), len(f)))
    assert T.nnz > 0
    C = H @ T - T @ H
    assert abs(C).max() <= 1e-12 * abs(H).max() * abs(T).max()


@pytest.mark.parametrize("N,norb0,tlz", [(3, 5, 0), (4, 6, -2), (5, 6, 1), (6, 9, 0)])
def test_c_restatement_matches_python(oracle, N, norb0, tlz):
    """oracle.c's two-level basis and build (the CPU baseline) agree bit for
    bit with the Python loops."""
    n1 = norb0 + 2
    f, s = oracle.basis2(N, norb0, tlz)
    words = np.array([(int(a) << n1) | int(b) for a, b in zip(f, s)], dtype=np.uint64)
    assert np.array_equal(oracle.basis2_c(N, norb0, tlz), words)
    kt0, vt0 = oracle.quartic_tables(norb0, oracle.odd_coulomb_list(norb0))
    kt1, vt1 = oracle.quartic_tables(n1, np.random.default_rng(2).uniform(-1, 2, n1 - 1))
    e0, e1 = np.linspace(-0.3, 0.3, norb0), np.full(n1, 0.7)
    a = oracle.build_upper2(f, s, norb0, kt0, vt0, kt1, vt1, e0, e1)
    b = oracle.build_upper2_c(words, norb0, kt0, vt0, kt1, vt1, e0, e1, nthreads=2)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(a[2].view(np.uint64), b[2].view(np.uint64))
