"""GPU replay of TreeCorr's own Python layer against this module.

Each log (tests/golden/api_*.npz) holds the exact `_treecorr` calls TreeCorr's unchanged
Python made while a scenario ran through its public API on the reference's compiled module:
Catalog construction with k-means patches (KMeansInitTree, KMeansRun, KMeansAssign,
GenerateXYZ), GGCorrelation / NNCorrelation / KKCorrelation / GGGCorrelation process calls
(including the per-patch-pair calls and triviallyZero of a jackknife run, and an exact-mode
KK), with the arguments, the aliased output arrays before and after each call and the return
values.  The test replays every call on treecorr_gb300._treecorr in the same order with the
same arguments and compares each call's outputs with the reference's; then it gives the
replayed outputs to the Python-level steps the log's final results came from (the xi
finalisation, the jackknife covariance on the GPU) and compares with those results.
"""
import numpy as np
import pytest

import api_trace as A

pytestmark = pytest.mark.gpu
RTOL = 1e-5


@pytest.mark.parametrize("name", A.SCENARIOS)
def test_replay_boundary_calls(gpu_lib, name):
    T = gpu_lib
    tr = A.Trace(name)
    problems, _ = A.replay(T, tr, rtol=RTOL, out_names=A.corr2_out_names(tr))
    assert not problems, "\n".join(problems[:20])


def test_replay_final_results(gpu_lib):
    """The Python layer's results from the replayed outputs: xi+- of the flat GG scenario and
    xi of the exact-mode KK scenario (finalisation), and the jackknife covariance of the
    patch scenario (tc_jackknife_cov from the replayed per-patch-pair results)."""
    T = gpu_lib
    for name, keys in (("gg_flat", (("xip", "xi0"), ("xim", "xi2"), ("xip_im", "xi1"),
                                    ("xim_im", "xi3"))),
                       ("kk_exact", (("xi", "xi0"),))):
        tr = A.Trace(name)
        names = A.corr2_out_names(tr)
        _, incs = A.replay(T, tr, rtol=RTOL, out_names=names)
        last = max(incs)
        cid = next(e["id"] for e in tr.events if e["op"] == "new" and e["id"] in names)
        # One process call: the increment is the whole result.
        o = dict(zip(names[cid], incs[last]))
        for k, q in keys:
            got = A.finalize_xi(o[q], o["weight"])
            ref = tr.final[k]
            assert np.abs(got - ref).max() <= RTOL * np.abs(ref).max(), (name, k)
        assert np.array_equal(o["npairs"], tr.final["npairs"]), name
    tr = A.Trace("gg_sphere_jk")
    _, incs = A.replay(T, tr, rtol=RTOL, out_names=A.corr2_out_names(tr))
    pairs, res = A.patch_pairs(tr, incs)
    npatch = int(tr.final["patch"].max()) + 1
    v, cov = T.jackknife_cov(res, pairs, npatch, 2, cross_patch_weight="simple")
    ref = tr.final["cov"]
    assert np.abs(cov - ref).max() <= RTOL * np.abs(ref).max()
    w = res[:, 0].sum(axis=0)
    xip = A.finalize_xi(res[:, 3].sum(axis=0), w)
    assert np.abs(xip - tr.final["xip"]).max() <= RTOL * np.abs(tr.final["xip"]).max()
