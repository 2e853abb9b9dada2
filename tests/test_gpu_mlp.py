"""Warm-start MLP (K10/K11): device forward and gradients against the FP64
oracle (oracle/mlp_oracle.py, bfloat16 at the same points), training, and
what the trained network gains over a random start."""
import numpy as np
import pytest

import hamiltonian_diagonalization_gb300 as ed
from oracle import mlp_oracle as MO

pytestmark = pytest.mark.gpu


def sample(torch, norb, N, m, seed):
    from oracle import oracle as O
    b = O.basis(N, norb, 0)
    rng = np.random.default_rng(seed)
    words = b[rng.integers(0, len(b), m)]
    v1 = rng.uniform(0.5, 3.0, m).astype(np.float32)
    target = np.stack([rng.normal(-6, 2, m), rng.integers(0, 2, m)], 1).astype(np.float32)
    dev = (torch.from_numpy(words.view(np.int64)).cuda(), torch.from_numpy(v1).cuda(),
           torch.from_numpy(np.ascontiguousarray(target)).cuda())
    return words, v1, target, dev


def test_forward_matches_oracle(cuda):
    torch = cuda
    net = ed.WarmStartMLP(22, 256, seed=3)
    words, v1, _, (wd, vd, _) = sample(torch, 22, 8, 1000, 1)
    out = torch.empty((1000, 8), dtype=torch.float32, device="cuda")
    net.forward(wd, vd, out)
    torch.cuda.synchronize()
    Zs, _ = MO.forward(net.params(), words, v1, 22, 256)
    got = out.cpu().numpy()[:, :2]
    ref = Zs[3][:, :2]
    assert np.max(np.abs(got - ref)) <= 1e-3 * max(1.0, np.max(np.abs(ref)))


def test_gradients_match_oracle(cuda):
    torch = cuda
    norb, H = 22, 128
    net = ed.WarmStartMLP(norb, H, seed=7)
    words, v1, target, (wd, vd, td) = sample(torch, norb, 8, 300, 2)
    g, loss = net.gradients(wd, vd, td)
    lref, gref = MO.loss_and_grads(net.params(), words, v1, target, norb, H)
    assert abs(loss - lref) <= 1e-4 * abs(lref)
    dims, offs, _ = MO.layout(norb, H)
    for l, (w, b) in enumerate(offs):
        for lo, hi in ((w, b), (b, b + dims[l + 1])):
            ref = gref[lo:hi]
            err = np.linalg.norm(g[lo:hi] - ref) / max(np.linalg.norm(ref), 1e-30)
            assert err < 2e-2, (l, lo, err)


def ground_states(torch, basis, norb, v1s, nev=1, seed=0):
    base = ed.odd_coulomb_list(norb)
    lists = []
    for v in v1s:
        x = base.copy()
        x[1] = v
        lists.append(x)
    batch = ed.HamiltonianBatch(basis, lists, autotune=False)
    ev, vec, info = batch.solve(nev, tol=1e-10, seed=seed, want_vectors=True)
    return batch, ev, vec, info


def test_training_and_warm_start_gain(cuda):
    torch = cuda
    N, norb = 8, 22
    basis = ed.FermionFockBasis()
    basis.GenerateFockSpace(N, norb, 0)
    v1_all = np.linspace(0.5, 3.0, 16)
    held = v1_all[[3, 7, 11, 14]]
    train = np.array([v for v in v1_all if v not in held])
    _, ev_tr, vec_tr, _ = ground_states(torch, basis, norb, train)
    psi = vec_tr[0].contiguous()                      # [n][len(train)] ground states
    net = ed.WarmStartMLP(norb, 256, seed=1)
    loss0 = net.fit(basis, train, psi, steps=1, batch=2048, lr=1e-3, seed=9)
    loss1 = net.fit(basis, train, psi, steps=1500, batch=2048, lr=1e-3, seed=10)
    assert loss1 < 0.5 * loss0
    n = basis.GetStoredDimension()
    V0 = torch.empty((n, len(held)), dtype=torch.float64, device="cuda")
    net.warm_start(basis, held, V0)
    batch, ev_rand, vec_true, info_rand = ground_states(torch, basis, norb, held, seed=4)
    ev_warm, _, info_warm = batch.solve(1, tol=1e-10, V0=V0)
    assert np.max(np.abs(ev_warm - ev_rand) / np.abs(ev_rand)) <= 1e-10
    # overlap of the predicted state with the converged ground state
    P = V0.cpu().numpy()
    T = vec_true[0].cpu().numpy()
    ov = np.abs(np.sum(P * T, axis=0)) / np.linalg.norm(P, axis=0)
    assert np.min(ov) > 0.5, ov
    assert info_warm["block_products"] < info_rand["block_products"], (info_warm, info_rand)
    # warm-started ground energies against the FP64 oracle (CPU build + ARPACK)
    from oracle import oracle as O
    words = O.basis(N, norb, 0)
    for j, v1 in enumerate(held):
        kt, vt = O.quartic_tables(norb, O.sweep_list(norb, v1))
        rp, col, val = O.build_upper(words, norb, kt, vt)
        e0 = O.lowest_eigenpairs(rp, col, val, 1, tol=1e-12)[0][0]
        assert abs(ev_warm[j, 0] - e0) <= 1e-10 * abs(e0), (j, ev_warm[j, 0], e0)
