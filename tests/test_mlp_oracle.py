"""The MLP oracle's building blocks on the CPU: bfloat16 rounding matches
torch's round-to-nearest-even conversion, and the oracle's gradient matches a
finite difference of its own loss (with bfloat16 rounding switched off)."""
import numpy as np

from oracle import mlp_oracle as MO


def test_bf16_rounding_matches_torch():
    import torch
    x = np.random.default_rng(0).standard_normal(100000).astype(np.float32) * 10
    x[:4] = [1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 0.0]
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(MO.bf16(x), ref)


def test_oracle_gradient_by_finite_differences(monkeypatch):
    monkeypatch.setattr(MO, "bf16", lambda v: np.asarray(v, dtype=np.float64))
    norb, H = 10, 64
    rng = np.random.default_rng(1)
    _, _, nparam = MO.layout(norb, H)
    p = rng.uniform(-0.2, 0.2, nparam)
    words = rng.integers(0, 1 << norb, 20).astype(np.uint64)
    v1 = rng.uniform(0.5, 3.0, 20)
    target = np.stack([rng.normal(-3, 1, 20), rng.integers(0, 2, 20)], 1)
    loss, g = MO.loss_and_grads(p, words, v1, target, norb, H)
    for i in rng.choice(nparam, 25, replace=False):
        e = np.zeros(nparam)
        e[i] = 1e-6
        lp, _ = MO.loss_and_grads(p + e, words, v1, target, norb, H)
        lm, _ = MO.loss_and_grads(p - e, words, v1, target, norb, H)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])
