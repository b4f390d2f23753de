"""GPU checks of the learned opening criterion: the training kernel's gradient against the
CPU oracle, the traversal's FP16 tensor-core evaluation against its emulation, and the
training pairs collected by a traversal."""
import os
import sys

import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


def _params(seed, scale=0.2):
    rng = np.random.default_rng(seed)
    return rng.normal(0, scale, M.NPARAM).astype(np.float32)


def test_gradient_matches_oracle(gpu_lib):
    T = gpu_lib
    rng = np.random.default_rng(2)
    p = _params(2)
    x = rng.uniform(0, 1.5, (3000, M.NIN)).astype(np.float32)
    t = rng.normal(-3, 1, 3000).astype(np.float32)
    g, loss = T.mlp_grad(p, x, t)
    g0, loss0 = M.grad(p.astype(np.float64), x.astype(np.float64), t.astype(np.float64))
    assert abs(loss - loss0) <= 1e-4 * abs(loss0)
    # FP32 arithmetic and atomics: compare relative to each block's largest gradient.
    offs = [0, 320, 384, 384 + 4096, 384 + 4096 + 64, 384 + 4096 + 128, M.NPARAM]
    for a, b in zip(offs[:-1], offs[1:]):
        scale = np.abs(g0[a:b]).max()
        assert np.abs(g[a:b] - g0[a:b]).max() <= 1e-4 * scale + 1e-7, (a, b)


def test_warp_inference_matches_fp16_emulation(gpu_lib):
    T = gpu_lib
    rng = np.random.default_rng(3)
    p = _params(3)
    x = np.stack([rng.uniform(1, 4, 1000), rng.uniform(0, 2, 1000), rng.uniform(0, 0.5, 1000),
                  rng.uniform(0, 1, 1000), np.full(1000, 0.19)], axis=1).astype(np.float32)
    y = T.mlp_infer(p, x)
    y0 = M.infer_fp16(p, x)
    assert np.all(np.isfinite(y))
    assert np.abs(y - y0).max() <= 2e-3 * (1 + np.abs(y0).max())


def test_training_reduces_loss(gpu_lib):
    T = gpu_lib
    from treecorr_gb300 import learned
    rng = np.random.default_rng(4)
    x = rng.uniform(0, 1, (20000, M.NIN)).astype(np.float32)
    t = (np.sin(3 * x[:, 0]) - 2 * x[:, 2] + 0.5 * x[:, 1] * x[:, 3] - 3).astype(np.float32)
    p, loss = learned.train(x, t, steps=600, batch=2048, lr=3e-3, seed=1)
    assert loss[-50:].mean() < 0.05 * loss[:10].mean()
    # The trained network, evaluated by the traversal's FP16 path, fits the data.
    y = T.mlp_infer(p, x[:2000])
    assert np.sqrt(((y - t[:2000]) ** 2).mean()) < 0.1


def test_collect_training_pairs(gpu_lib):
    T = gpu_lib
    import helpers as H
    from cases import flat_catalog
    rng = np.random.default_rng(5)
    cat = flat_catalog(rng, 40000, L=300.)
    nb, lo, hi = 20, 1.0, 100.0
    bs = np.log(hi / lo) / nb
    bins = dict(nbins=nb, min_sep=lo, max_sep=hi, bin_size=bs, b=0.1 * bs, a=0.1)
    out = {k: np.zeros(nb) for k in H.OUT_KEYS}
    corr = T.GGCorr(T.Log, lo, hi, nb, bs, 0.1 * bs, 0.1, -sys.float_info.max,
                    sys.float_info.max, 0., 0., 0., out["xi0"], out["xi1"], out["xi2"],
                    out["xi3"], out["meanr"], out["meanlogr"], out["weight"], out["npairs"])
    f = H.gpu_field(T, "G", "flat", cat, 0.0, 0.0)
    x, t = corr.learnCollect(f, T.Euclidean, sample_mod=4, max_samples=200000)
    assert len(t) > 1000
    ok = np.isfinite(t)
    assert ok.mean() > 0.5
    # Candidates are pairs the rule splits: sizes above b * r, below min(a, 4 b) * r.
    s_over_w = x[:, 0] + x[:, 1]          # (s1 + s2) / (r * bin_size)
    assert np.all(s_over_w * bs <= 4 * 0.1 * bs * (1 + 1e-4))
    assert np.all((x[:, 2] >= 0) & (x[:, 2] <= 0.5))
    assert np.all((t[ok] >= np.log10(1e-5) - 1e-4) & (t[ok] <= 1e-4))
    # The sampling traversal still computed the plain result.
    ref = {k: np.zeros(nb) for k in H.OUT_KEYS}
    c2 = T.GGCorr(T.Log, lo, hi, nb, bs, 0.1 * bs, 0.1, -sys.float_info.max,
                  sys.float_info.max, 0., 0., 0., ref["xi0"], ref["xi1"], ref["xi2"],
                  ref["xi3"], ref["meanr"], ref["meanlogr"], ref["weight"], ref["npairs"])
    c2.processAuto(f, False, False, T.Euclidean)
    assert np.array_equal(out["npairs"], ref["npairs"])
