"""The learned preconditioner's CPU oracle (no reference counterpart) is
pinned by finite differences: its backward is the exact gradient of its
forward (float64, bf16 rounding off)."""
import numpy as np

from oracle import unet


def _params(seed):
    rng = np.random.default_rng(seed)
    out = []
    for _, ci, co in unet.LAYERS:
        out += [rng.standard_normal(ci * co * 9) * np.sqrt(2.0 / (ci * 9)), rng.standard_normal(co) * 0.1]
    return np.concatenate(out)


def test_oracle_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = _params(1)
    x = rng.standard_normal((1, 2, 8, 16))
    dpred = rng.standard_normal((1, 8, 16))
    pred, cache = unet.forward(p, x, rounding=False)
    g = unet.backward(p, cache, dpred)
    assert g.shape == p.shape
    idx = rng.choice(p.size, 40, replace=False)
    eps = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += eps
        fp = np.sum(unet.forward(q, x, rounding=False)[0] * dpred)
        q[i] -= 2 * eps
        fm = np.sum(unet.forward(q, x, rounding=False)[0] * dpred)
        fd = (fp - fm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_bf16_rounding_is_round_to_nearest_even():
    import torch
    a = np.random.default_rng(2).standard_normal(10000).astype(np.float32) * 100
    want = torch.tensor(a).bfloat16().float().numpy().astype(np.float64)
    assert np.array_equal(unet._round(a), want)
