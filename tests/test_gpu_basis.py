"""Device Fock basis (K1) and rank (K2) against the reference's own scan
(golden digests) and the oracle's binary search: bit-exact."""
import hashlib
import json
import os

import numpy as np
import pytest

import hamiltonian_diagonalization_gb300 as ed

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
MISS = np.uint64(0xFFFFFFFFFFFFFFFF)


@pytest.fixture(scope="module")
def bases():
    with open(os.path.join(GOLD, "ref_bases.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("key", ["2_8_0", "4_10_0", "4_10_-2", "6_16_0", "6_16_4", "8_22_0", "8_22_2", "10_28_0",
                                 "10_28_2", "10_28_4", "10_28_6", "10_28_8", "11_31_0", "12_34_0"])
def test_basis_matches_reference(cuda, bases, key):
    ent = bases[key]
    b = ed.FermionFockBasis()
    empty = b.GenerateFockSpace(ent["N"], ent["norb"], ent["two_lz"])
    assert empty == (ent["dim"] == 0)
    words = b.GetFockBasis()
    assert len(words) == ent["dim"]
    assert hashlib.sha256(words.astype("<u8").tobytes()).hexdigest() == ent["sha256"]
    if "words" in ent:
        assert np.array_equal(words, np.array(ent["words"], dtype=np.uint64))
    # every basis word ranks to its own index
    idx = b.FindFockStateIndices(words)
    assert np.array_equal(idx, np.arange(len(words), dtype=np.uint64))


def test_rank_matches_binary_search_with_misses(cuda, oracle):
    rng = np.random.default_rng(11)
    for (N, norb, tlz) in [(8, 22, 0), (10, 28, 4), (5, 40, 3), (3, 17, -6)]:
        b = ed.FermionFockBasis()
        b.GenerateFockSpace(N, norb, tlz)
        ref = oracle.basis(N, norb, tlz)
        assert np.array_equal(b.GetFockBasis(), ref)
        # in-sector words, other-sector words, wrong popcount, bits above norb
        q = [ref[rng.integers(0, len(ref), 3000)]]
        other = oracle.basis(N, norb, tlz + 2)
        if len(other):
            q.append(other[rng.integers(0, len(other), 1000)])
        q.append(rng.integers(0, 1 << min(norb, 62), 1000, dtype=np.uint64))
        q.append(ref[:200] | np.uint64(1 << norb) if norb < 64 else ref[:0])
        q.append(np.array([0, 1, 2 ** 64 - 1], dtype=np.uint64))
        q = np.concatenate(q).astype(np.uint64)
        assert np.array_equal(b.FindFockStateIndices(q), oracle.find_indices(ref, q))


def test_edge_sectors(cuda, oracle):
    b = ed.FermionFockBasis()
    # odd parity and out-of-range sectors are empty, like isZeroDim
    assert b.GenerateFockSpace(4, 10, 1) is True and b.GetStoredDimension() == 0
    assert b.GenerateFockSpace(4, 10, 100) is True
    assert int(b.FindFockStateIndices(np.array([15], dtype=np.uint64))[0]) == int(MISS)
    # one particle, and a completely filled level (single state)
    for (N, norb, tlz) in [(1, 9, -8), (1, 9, 8), (9, 9, 0), (2, 2, 0), (1, 1, 0)]:
        b.GenerateFockSpace(N, norb, tlz)
        assert np.array_equal(b.GetFockBasis(), oracle.basis(N, norb, tlz))
    # the largest orbital count of the device path
    b.GenerateFockSpace(3, 40, 0)
    assert np.array_equal(b.GetFockBasis(), oracle.basis(3, 40, 0))
    with pytest.raises(ed.EDError):
        b.GenerateFockSpace(3, 41, 0)
