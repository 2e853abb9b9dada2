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
