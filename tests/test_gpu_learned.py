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


def _gg_corr(T, bins, out):
    return T.GGCorr(T.Log, bins["min_sep"], bins["max_sep"], bins["nbins"], bins["bin_size"],
                    bins["b"], bins["a"], -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
                    out["xi0"], out["xi1"], out["xi2"], out["xi3"], out["meanr"],
                    out["meanlogr"], out["weight"], out["npairs"])


def _flat_setup(T, n=40000, L=300., seed=5):
    import helpers as H
    from cases import flat_catalog
    cat = flat_catalog(np.random.default_rng(seed), n, L=L)
    nb, lo, hi = 20, 1.0, 100.0
    bs = np.log(hi / lo) / nb
    f = H.gpu_field(T, "G", "flat", cat, 0.0, 0.0)
    return cat, f, dict(nbins=nb, min_sep=lo, max_sep=hi, bin_size=bs, a=0.1)


def _run(T, f, bins, params=None, threshold=-3.0, cand_factor=4.0):
    import helpers as H
    out = {k: np.zeros(bins["nbins"]) for k in H.OUT_KEYS}
    c = _gg_corr(T, bins, out)
    if params is not None:
        c.setLearned(params, threshold=threshold, cand_factor=cand_factor)
    c.processAuto(f, False, False, T.Euclidean)
    out["_stats"] = c.stats()
    return out


def _xi_err(out, ref):
    """max over bins of |d xi+-| / max |xi+| (the metric's measure)."""
    xp, xm = out["xi0"] / out["weight"], out["xi2"] / out["weight"]
    rp, rm = ref["xi0"] / ref["weight"], ref["xi2"] / ref["weight"]
    mx = np.abs(rp).max()
    return max(np.abs(xp - rp).max(), np.abs(xm - rm).max()) / mx


def test_learned_traversal_accepting_nothing_is_plain(gpu_lib):
    """k_expand<2> with a threshold no prediction can meet: the network is evaluated on every
    candidate and accepts none, so the result is the bin_slop rule's (the reference's
    include/BinType.h:93-151)."""
    T = gpu_lib
    cat, f, bins = _flat_setup(T)
    bins = dict(bins, b=0.1 * bins["bin_size"])
    plain = _run(T, f, bins)
    learned = _run(T, f, bins, params=_params(7), threshold=-1e30)
    st = learned["_stats"]
    assert st["learned"] == 0
    assert st["cell_pairs"] == plain["_stats"]["cell_pairs"]
    assert np.array_equal(learned["npairs"], plain["npairs"])
    for k in ("weight", "xi0", "xi1", "xi2", "xi3", "meanr", "meanlogr"):
        np.testing.assert_allclose(learned[k], plain[k], rtol=1e-6,
                                   atol=1e-6 * np.abs(plain["weight"]).max())


def test_learned_traversal_error_and_gain(gpu_lib):
    """A network trained on this distribution's split candidates, used inside the traversal
    (base bin_slop 0.1, candidates up to 4 b r, accept when the predicted log10 leak <= -3),
    against the exact result (bin_slop 0, angle_slop 0) on the same catalog: its error lies
    between the base rule's and the rule at 4 b, and it evaluates fewer cell pairs than the
    base rule (what the network gains).  At bin_slop 0 -- the only setting whose error meets
    1e-4 of max|xi+| on shape-noise-dominated data -- the network has no candidates at all
    (they are pairs the rule splits within cand_factor * b * r), so it can gain nothing."""
    import time
    import torch
    T = gpu_lib
    from treecorr_gb300 import learned
    cat, f, bins = _flat_setup(T)
    bs = bins["bin_size"]
    # Training pairs from a separate catalog of the same distribution.
    _, ftrain, _ = _flat_setup(T, seed=55)
    out = {k: np.zeros(bins["nbins"]) for k in ("xi0", "xi1", "xi2", "xi3", "meanr",
                                                 "meanlogr", "weight", "npairs")}
    c = _gg_corr(T, dict(bins, b=0.1 * bs), out)
    x, y = learned.collect(c, ftrain, T.Euclidean, sample_mod=2, max_samples=400000)
    params, loss = learned.train(x, y, steps=1500, batch=4096, lr=2e-3, seed=0)
    exact = _run(T, f, dict(bins, b=0.0, a=0.0))
    base = _run(T, f, dict(bins, b=0.1 * bs))
    wide = _run(T, f, dict(bins, b=0.4 * bs))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lrn = _run(T, f, dict(bins, b=0.1 * bs), params=params, threshold=-3.0, cand_factor=4.0)
    t_lrn = time.perf_counter() - t0
    t0 = time.perf_counter()
    base2 = _run(T, f, dict(bins, b=0.1 * bs))
    t_base = time.perf_counter() - t0
    e_base, e_wide, e_lrn = _xi_err(base, exact), _xi_err(wide, exact), _xi_err(lrn, exact)
    st = lrn["_stats"]
    gain = base2["_stats"]["cell_pairs"] / st["cell_pairs"]
    print(f"xi err: base {e_base:.3e}  learned {e_lrn:.3e}  4b {e_wide:.3e}; cell pairs "
          f"base {base2['_stats']['cell_pairs']} learned {st['cell_pairs']} (gain {gain:.3f}, "
          f"{st['learned']} accepted by the network); wall base {t_base:.3f} s learned "
          f"{t_lrn:.3f} s")
    assert st["learned"] > 0
    assert st["cell_pairs"] < base2["_stats"]["cell_pairs"]
    assert e_lrn <= 1.5 * e_wide + 1e-6
    # Exact mode: nothing is a candidate, so the network changes nothing.
    ex_l = _run(T, f, dict(bins, b=0.0, a=0.0), params=params, threshold=10.0)
    assert ex_l["_stats"]["learned"] == 0
    assert np.array_equal(ex_l["npairs"], exact["npairs"])
