"""Shared-subspace sweep (eigenvector continuation): subset solves of a batch,
the subspace's Gram-Schmidt, the Ritz step of every Hamiltonian of a batch,
and the continuation sweep against the oracle's Hamiltonians."""
import numpy as np
import pytest

import hamiltonian_diagonalization_gb300 as ed
from hamiltonian_diagonalization_gb300.sweep import solve_sector_subspace, sweep_lists

pytestmark = pytest.mark.gpu


def oracle_lowest(oracle, N, norb, tlz, pp, k):
    """Lowest k eigenvalues of the oracle's Hamiltonian (restated reference
    build, full symmetric matrix) by ARPACK."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    b = oracle.basis(N, norb, tlz)
    kt, vt = oracle.quartic_tables(norb, pp)
    rp, col, val = oracle.build_upper(b, norb, kt, vt)
    n = len(b)
    U = sp.csr_matrix((val, col, rp), shape=(n, n))
    H = (U + U.T - sp.diags(U.diagonal())).tocsr()
    v0 = np.random.default_rng(11).uniform(-1.0, 1.0, n)   # reaches both Lz-reflection parities
    w = sla.eigsh(H, k=k, which="SA", tol=1e-13, ncv=40, v0=v0, return_eigenvectors=False)
    return np.sort(w)


def test_subset_solve_matches_full_solve(cuda):
    N, norb, tlz, nev = 8, 22, 2, 4
    lists = sweep_lists(norb, [0.5, 0.9, 1.3, 1.9, 2.4, 3.0])
    b = ed.FermionFockBasis()
    b.GenerateFockSpace(N, norb, tlz)
    batch = ed.HamiltonianBatch(b, lists)
    ev, _, info = batch.solve(nev, tol=1e-10, seed=3)
    sel = [4, 1]
    evs, vec, infs = batch.solve(nev, tol=1e-10, seed=7, want_vectors=True, select=sel)
    assert vec.shape == (nev, batch.n, 2)
    assert infs["converged"] == 2 and infs["max_residual"] <= 1e-10
    assert np.max(np.abs(evs - ev[sel]) / np.abs(ev[sel])) <= 1e-10


def test_ritz_reproduces_solved_pairs(cuda):
    torch = cuda
    N, norb, tlz, nev = 8, 22, 0, 4
    lists = sweep_lists(norb, [0.6, 1.2, 2.0, 2.8])
    b = ed.FermionFockBasis()
    b.GenerateFockSpace(N, norb, tlz)
    batch = ed.HamiltonianBatch(b, lists)
    ev, vec, _ = batch.solve(nev, tol=1e-11, seed=1, want_vectors=True)
    sp = ed.Subspace(batch.n, 64)
    assert sp.add(vec) == nev * len(lists)
    # the same vectors again add nothing
    assert sp.add(vec) == 0 and sp.dim == nev * len(lists)
    evr, X, res = batch.subspace_ritz(sp, nev)
    assert X.shape == (nev, batch.n, len(lists))
    assert np.max(np.abs(evr - ev) / np.abs(ev)) <= 1e-12
    assert np.max(res) <= 1e-10
    # Ritz vectors are unit vectors
    nrm = torch.linalg.vector_norm(X, dim=1).cpu().numpy()
    assert np.max(np.abs(nrm - 1.0)) <= 1e-12


def test_ritz_rejects_a_family_of_too_high_rank(cuda):
    # ten lists scaling the ten odd-m pseudopotentials independently: rank 10
    N, norb, tlz = 6, 22, 0
    rng = np.random.default_rng(4)
    base = ed.odd_coulomb_list(norb)
    lists = []
    for _ in range(10):
        v = base.copy()
        v[1::2] *= rng.uniform(0.5, 1.5, len(v[1::2]))
        lists.append(v)
    b = ed.FermionFockBasis()
    b.GenerateFockSpace(N, norb, tlz)
    batch = ed.HamiltonianBatch(b, lists)
    _, vec, _ = batch.solve(2, tol=1e-10, seed=1, want_vectors=True, select=[0, 1])
    sp = ed.Subspace(batch.n, 8)
    sp.add(vec)
    with pytest.raises(ed.EDError):
        batch.subspace_ritz(sp, 2)


@pytest.mark.parametrize("tlz", [0, 4])
def test_subspace_sweep_matches_oracle(cuda, oracle, tlz):
    N, norb, nev, npts = 8, 22, 4, 24
    v1s = np.linspace(0.5, 3.0, npts)
    lists = sweep_lists(norb, v1s)
    b = ed.FermionFockBasis()
    b.GenerateFockSpace(N, norb, tlz)
    ev, rec = solve_sector_subspace(b, lists, nev, 1e-10, 1)
    assert not np.any(np.isnan(ev))
    assert rec["ritz_accepted"] > 0
    for j in range(npts):
        ref = oracle_lowest(oracle, N, norb, tlz, lists[j], nev)
        assert np.max(np.abs(ev[j] - ref) / np.abs(ref)) <= 1e-10, (j, ev[j], ref)
