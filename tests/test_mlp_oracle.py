"""The CPU oracle of the learned criterion's network: its gradient against central
finite differences (float64)."""
import numpy as np

from oracle import mlp_oracle as M


def test_oracle_gradient_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, M.NPARAM)
    x = rng.normal(0, 1, (50, M.NIN))
    t = rng.normal(0, 1, 50)
    g, loss = M.grad(p, x, t)
    assert np.isclose(loss, ((M.forward(p, x) - t) ** 2).mean())
    eps = 1e-6
    for i in rng.choice(M.NPARAM, 40, replace=False):
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (((M.forward(pp, x) - t) ** 2).mean() - ((M.forward(pm, x) - t) ** 2).mean()) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_fp16_emulation_close_to_fp64():
    rng = np.random.default_rng(1)
    p = rng.normal(0, 0.2, M.NPARAM)
    x = rng.uniform(0, 1, (64, M.NIN))
    assert np.allclose(M.infer_fp16(p, x), M.forward(p, x), rtol=2e-2, atol=2e-2)
