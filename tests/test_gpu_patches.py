"""Patch pairs in one expansion against one GPU call per pair, and the device jackknife
covariance against the CPU restatement of TreeCorr's (oracle/jackknife_oracle.py)."""
import sys

import numpy as np
import pytest

import helpers as H
from oracle import jackknife_oracle as J

pytestmark = pytest.mark.gpu


def _patches(seed=7, n=30000, npatch=6, L=200.):
    from cases import flat_catalog
    rng = np.random.default_rng(seed)
    cat = flat_catalog(rng, n, L=L)
    # Patches: nearest of npatch random centres (uneven sizes).
    cen = rng.uniform(0, L, (npatch, 2))
    d = (cat["x"][:, None] - cen[:, 0]) ** 2 + (cat["y"][:, None] - cen[:, 1]) ** 2
    pid = d.argmin(axis=1)
    return cat, pid, npatch


def _corr(T, out, nb, lo, hi, bs):
    return T.GGCorr(T.Log, lo, hi, nb, bs, 0.1 * bs, 0.1, -sys.float_info.max, sys.float_info.max,
                    0., 0., 0., out["xi0"], out["xi1"], out["xi2"], out["xi3"], out["meanr"],
                    out["meanlogr"], out["weight"], out["npairs"])


def test_patch_pairs_match_single_calls(gpu_lib):
    T = gpu_lib
    cat, pid, npatch = _patches()
    nb, lo, hi = 15, 1.0, 60.0
    bs = np.log(hi / lo) / nb
    sub = [{k: np.ascontiguousarray(v[pid == p]) for k, v in cat.items() if v is not None}
           for p in range(npatch)]
    fields = [H.gpu_field(T, "G", "flat", s, 0.0, 0.0) for s in sub]
    out = {k: np.zeros(nb) for k in H.OUT_KEYS}
    corr = _corr(T, out, nb, lo, hi, bs)
    pairs, res = corr.processPatches(fields, T.Euclidean)
    assert len(pairs) >= npatch
    keys = ("weight", "meanr", "meanlogr", "xi0", "xi1", "xi2", "xi3", "npairs")
    for (i, j), r in zip(pairs, res):
        o = {k: np.zeros(nb) for k in H.OUT_KEYS}
        c = _corr(T, o, nb, lo, hi, bs)
        if i == j:
            c.processAuto(fields[i], False, False, T.Euclidean)
        else:
            c.processCross(fields[i], fields[j], False, False, T.Euclidean)
        for q, k in enumerate(keys):
            ref = o[k]
            if k == "npairs":
                assert np.array_equal(r[q], ref), (i, j)
            else:
                # FP32 partial sums grouped differently (warps see other mixes of pairs):
                # the xi sums cancel, so they are compared against their largest bin.
                tol = 1e-6 if k.startswith("xi") else 1e-8
                assert np.allclose(r[q], ref, rtol=tol, atol=tol * np.abs(ref).max()), (i, j, k)


@pytest.mark.parametrize("cpw", ["simple", "mean", "match"])
def test_jackknife_matches_restatement(gpu_lib, cpw):
    T = gpu_lib
    cat, pid, npatch = _patches(seed=8, npatch=8)
    nb, lo, hi = 12, 1.0, 50.0
    bs = np.log(hi / lo) / nb
    sub = [{k: np.ascontiguousarray(v[pid == p]) for k, v in cat.items() if v is not None}
           for p in range(npatch)]
    fields = [H.gpu_field(T, "G", "flat", s, 0.0, 0.0) for s in sub]
    out = {k: np.zeros(nb) for k in H.OUT_KEYS}
    pairs, res = _corr(T, out, nb, lo, hi, bs).processPatches(fields, T.Euclidean)
    v, cov = T.jackknife_cov(res, pairs, npatch, 2, cpw)
    v0 = J.design_matrix(res, pairs, npatch, gg=True, cpw=cpw)
    c0 = J.cov_jackknife(v0)
    assert np.allclose(v, v0, rtol=1e-12, atol=1e-18)
    assert np.allclose(cov, c0, rtol=1e-10, atol=1e-22)
