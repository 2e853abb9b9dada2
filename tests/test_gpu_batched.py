"""Batched sweep (K6): the shared-pattern block product and the lockstep
Lanczos against the single-Hamiltonian path on the same inputs."""
import numpy as np
import pytest

import hamiltonian_diagonalization_gb300 as ed

pytestmark = pytest.mark.gpu


def sweep_lists(norb, v1s):
    base = ed.odd_coulomb_list(norb)
    out = []
    for v1 in v1s:
        v = base.copy()
        v[1] = v1
        out.append(v)
    return out


def single_product(torch, N, norb, tlz, pp, x):
    H = ed.SpinlessFermionHamiltonian()
    H.Initialize(N, norb, twoLz=tlz)
    H.Add_CdCdCC_Terms(ed.QuarticTermTables(norb, pp))
    xd = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    yd = torch.empty_like(xd)
    ed.MatrixVectorFunction(H).Simple(xd, yd)
    torch.cuda.synchronize()
    return yd.cpu().numpy()


@pytest.mark.parametrize("case", [(6, 16, 4), (8, 22, 0)])
def test_block_product_matches_single_products(cuda, case):
    torch = cuda
    N, norb, tlz = case
    lists = sweep_lists(norb, [0.5, 1.1, 2.0, 3.0, 0.8])
    b = ed.FermionFockBasis()
    b.GenerateFockSpace(N, norb, tlz)
    batch = ed.HamiltonianBatch(b, lists)
    n, B = batch.n, batch.nham
    X = np.random.default_rng(2).uniform(-1, 1, (n, B))
    Xd = torch.from_numpy(X).cuda()
    Yd = torch.empty_like(Xd)
    batch.spmm(Xd, Yd)
    torch.cuda.synchronize()
    Y = Yd.cpu().numpy()
    for j, pp in enumerate(lists):
        y = single_product(torch, N, norb, tlz, pp, X[:, j])
        assert np.max(np.abs(Y[:, j] - y)) <= 1e-13 * np.max(np.abs(y)), j


def test_batched_solve_matches_single_solves(cuda):
    torch = cuda
    N, norb, tlz, nev = 8, 22, 0, 4
    v1s = [0.6, 1.4, 2.2, 2.9]
    lists = sweep_lists(norb, v1s)
    b = ed.FermionFockBasis()
    b.GenerateFockSpace(N, norb, tlz)
    batch = ed.HamiltonianBatch(b, lists)
    ev, vec, info = batch.solve(nev, tol=1e-10, seed=5, want_vectors=True)
    assert info["converged"] == len(v1s), info
    assert info["max_residual"] <= 1e-10
    assert info["tile_hamiltonians"] in (4, 8, 16, 32) and info["tile_l1"] in (0, 1)
    for j, pp in enumerate(lists):
        out = ed.solve_sector(N, norb, tlz, pp, nev, tol=1e-10, seed=11)
        assert np.max(np.abs(ev[j] - out["eigenvalues"]) / np.abs(out["eigenvalues"])) <= 1e-10, j
    # eigenvectors: unit norm, orthogonal within each Hamiltonian
    V = vec.cpu().numpy()          # [nev, n, nham]
    for j in range(len(v1s)):
        G = V[:, :, j] @ V[:, :, j].T
        assert np.max(np.abs(G - np.eye(nev))) < 1e-9


def test_batched_solve_from_given_starts(cuda):
    torch = cuda
    N, norb, tlz = 6, 16, 0
    lists = sweep_lists(norb, [1.0, 2.0])
    b = ed.FermionFockBasis()
    b.GenerateFockSpace(N, norb, tlz)
    batch = ed.HamiltonianBatch(b, lists, autotune=False)
    V0 = torch.from_numpy(np.random.default_rng(0).uniform(-1, 1, (batch.n, 2))).cuda()
    ev, _, info = batch.solve(2, tol=1e-10, V0=V0)
    assert info["converged"] == 2
    with pytest.raises(ed.EDError):
        batch.solve(2, V0=torch.zeros((batch.n, 2), dtype=torch.float64, device="cuda"))


def test_converged_hamiltonians_retire_from_the_batch(cuda):
    """A Hamiltonian that converges restarts ahead of the others leaves the
    batch; its eigenpairs (written at retirement) and the survivors' match
    one-at-a-time solves from the same start vectors."""
    torch = cuda
    N, norb, tlz, nev = 10, 28, 0, 4
    v1s = [0.5, 2.1, 2.9]
    lists = sweep_lists(norb, v1s)
    b = ed.FermionFockBasis()
    b.GenerateFockSpace(N, norb, tlz)
    n = b.GetStoredDimension()
    rng = np.random.default_rng(7)
    V0 = rng.uniform(-1, 1, (n, len(v1s)))
    # Hamiltonian 1 starts next to its own lowest states (1e-3 of random left,
    # so the Krylov space is not exactly invariant): it converges early
    near = ed.solve_sector(N, norb, tlz, lists[1], nev, tol=1e-10, seed=3, want_vectors=True)["eigenvectors"]
    r = rng.uniform(-1, 1, n)
    V0[:, 1] = near.sum(axis=0) + 1e-3 * r / np.linalg.norm(r)
    batch = ed.HamiltonianBatch(b, lists, autotune=False)
    ev, vec, info = batch.solve(nev, tol=1e-10, V0=torch.from_numpy(np.ascontiguousarray(V0)).cuda(),
                                want_vectors=True)
    assert info["converged"] == len(v1s) and info["max_residual"] <= 1e-10
    # retirement: fewer Hamiltonian-products than block products x batch size
    assert info["problem_products"] < info["block_products"] * len(v1s), info
    V = vec.cpu().numpy()                # [nev, n, nham]
    for j, pp in enumerate(lists):
        out = ed.solve_sector(N, norb, tlz, pp, nev, tol=1e-10, v0=V0[:, j], want_vectors=True)
        assert np.max(np.abs(ev[j] - out["eigenvalues"]) / np.abs(out["eigenvalues"])) <= 1e-10, j
        G = V[:, :, j] @ V[:, :, j].T
        assert np.max(np.abs(G - np.eye(nev))) < 1e-9, j
        # same eigenvectors up to sign (the levels are not degenerate here)
        ov = np.abs(np.sum(V[:, :, j] * out["eigenvectors"], axis=1))
        assert np.min(ov) > 1 - 1e-8, (j, ov)


def test_continuation_sweep_matches_random_starts(cuda):
    # anchors from random starts, the rest from their nearest anchor's states:
    # the same eigenvalues as random starts, in fewer products
    from hamiltonian_diagonalization_gb300 import sweep
    N, norb, nev = 8, 22, 3
    v1s = np.linspace(0.5, 3.0, 16)
    tc, ec, rec = sweep.run_continuation(N, norb, [0], v1s, nev, 1e-10, 1)
    tb, eb, infos = sweep.run_batched(N, norb, [0], v1s, nev, 1e-10, 1)
    assert sorted(ec) == sorted(eb)
    for k in eb:
        assert np.max(np.abs(ec[k] - eb[k]) / np.abs(eb[k])) <= 1e-10, k
    r = rec[0]
    assert r["anchors"] + r["warm_points"] == len(v1s)
    per_warm = r["warm_problem_products"] / r["warm_points"]
    per_random = infos[0]["problem_products"] / len(v1s)
    assert per_warm < per_random, (per_warm, per_random)


@pytest.mark.parametrize("case", [(8, 22, 4), (9, 24, 1), (7, 19, 0)])
def test_batched_solve_matches_oracle(cuda, oracle, case):
    # the batch's eigenvalues against the oracle's Hamiltonians (the reference's
    # quartic build restated, pinned to the compiled reference), solved by
    # SciPy's ARPACK from a random start that reaches both Lz-reflection parities
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    N, norb, tlz = case
    nev = 4
    v1s = [0.4, 1.1, 2.3, 3.0]
    lists = sweep_lists(norb, v1s)
    basis = ed.FermionFockBasis()
    basis.GenerateFockSpace(N, norb, tlz)
    batch = ed.HamiltonianBatch(basis, lists)
    ev, _, info = batch.solve(nev, tol=1e-10, seed=4)
    assert info["converged"] == len(v1s) and info["max_residual"] <= 1e-10
    b = oracle.basis(N, norb, tlz)
    v0 = np.random.default_rng(12).uniform(-1.0, 1.0, len(b))
    for j, pp in enumerate(lists):
        kt, vt = oracle.quartic_tables(norb, pp)
        rp, col, val = oracle.build_upper(b, norb, kt, vt)
        U = sp.csr_matrix((val, col, rp), shape=(len(b), len(b)))
        H = (U + U.T - sp.diags(U.diagonal())).tocsr()
        ref = np.sort(sla.eigsh(H, k=nev, which="SA", tol=1e-13, ncv=40, v0=v0, return_eigenvectors=False))
        assert np.max(np.abs(ev[j] - ref) / np.abs(ref)) <= 1e-10, (j, ev[j], ref)
