"""Learned warm start of the matrix-free solve: the network retrained on a
sector's ground states along the V1 sweep seeds the matrix-free Lanczos of
that sector's Coulomb Hamiltonian, with the random start as the fallback."""
import numpy as np
import pytest

import hamiltonian_diagonalization_gb300 as ed
from hamiltonian_diagonalization_gb300.sweep import matfree_warm_start, warm_started_solve

pytestmark = pytest.mark.gpu


def test_retrained_network_cuts_matrix_free_products(cuda):
    # N=10, 2S=27, Lz=0 (246,448 states): trained on six sweep points
    # 0.5 ... 0.90, predicting the Coulomb V1 = 0.4626
    rec = matfree_warm_start(10, 28, 0, nevs=(1, 3), steps=6000, seed=1)
    assert rec["prediction_finite"]
    for nev, res in rec["solves"].items():
        ref = np.array(res["eigenvalues"])
        for name, r in res.items():
            if not isinstance(r, dict):
                continue
            assert r["max_residual"] <= 1e-10, (nev, name)
            if name != "random":
                assert not r["fallback"], (nev, name)
                assert r["max_rel_eig_diff"] <= 1e-10, (nev, name)
    one = rec["solves"]["1"]
    assert one["mlp_mix0"]["overlap"] > 0.5
    assert one["mlp_mix0"]["products"] < one["random"]["products"]
    assert one["nearest"]["products"] < one["random"]["products"]


def test_warm_start_falls_back_to_random(cuda):
    N, norb, tlz, nev = 8, 22, 0, 3
    pp = ed.odd_coulomb_list(norb)
    ref = ed.solve_sector(N, norb, tlz, pp, nev, tol=1e-10, seed=5, matrix_free=True)
    b = ed.FermionFockBasis()
    b.GenerateFockSpace(N, norb, tlz)
    n = b.GetStoredDimension()
    for bad in (None, np.zeros(n), np.full(n, np.nan)):
        out, fallback = warm_started_solve(N, norb, tlz, pp, nev, bad, seed=5)
        assert fallback
        assert np.max(np.abs(out["eigenvalues"] - ref["eigenvalues"]) / np.abs(ref["eigenvalues"])) <= 1e-12
    # a good start is used as given, mixed with the random start for nev > 1
    out, fallback = warm_started_solve(N, norb, tlz, pp, nev, np.ones(n), seed=5)
    assert not fallback
    assert np.max(np.abs(out["eigenvalues"] - ref["eigenvalues"]) / np.abs(ref["eigenvalues"])) <= 1e-10
