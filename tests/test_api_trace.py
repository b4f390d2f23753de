"""CPU checks of the `_treecorr` call logs of TreeCorr's own Python layer (tests/api_trace.py):
the replacement module exposes every class, function and method the logs use, each with a
signature that accepts the logged arguments; the logged results are consistent with the
reference's Python finalisation; and the oracle's jackknife restatement gives the reference
Python's covariance from the logged per-patch-pair results (treecorr/corr2base.py:1787-1823,
2432-2445)."""
import inspect

import numpy as np
import pytest

import api_trace as A


@pytest.mark.parametrize("name", A.SCENARIOS)
def test_module_accepts_every_logged_call(name):
    from treecorr_gb300 import _treecorr as T
    tr = A.Trace(name)
    classes = {}
    for e in tr.events:
        if e["op"] == "new":
            cls = getattr(T, e["cls"])
            inspect.signature(cls).bind(*e["args"])
            classes[e["id"]] = cls
        elif e["op"] == "fn":
            inspect.signature(getattr(T, e["name"])).bind(*e["args"])
        else:
            meth = getattr(classes[e["id"]], e["method"])
            inspect.signature(meth).bind(None, *e["args"])
        for a in e.get("args", []):
            if isinstance(a, dict) and "enum" in a:
                assert hasattr(T, a["name"]), a


def test_logged_results_match_the_python_finalisation():
    """xip = xi0 / weight etc. (the reference's _finalize) on the logged final outputs gives
    the Python layer's logged results: the boundary outputs alone determine them."""
    tr = A.Trace("gg_flat")
    names = A.corr2_out_names(tr)
    (cid, outs), = A.final_outs(tr).items()
    o = dict(zip(names[cid], outs))
    for k, q in (("xip", "xi0"), ("xip_im", "xi1"), ("xim", "xi2"), ("xim_im", "xi3")):
        np.testing.assert_allclose(A.finalize_xi(o[q], o["weight"]), tr.final[k], rtol=1e-12)
    np.testing.assert_array_equal(o["npairs"], tr.final["npairs"])


def test_jackknife_restatement_matches_reference_python():
    """The per-patch-pair results logged in the jackknife scenario, combined by the oracle's
    restatement of the jackknife (simple cross-patch weights, the scenario's), give the
    covariance and xi that TreeCorr's Python computed."""
    from oracle import jackknife_oracle as J
    tr = A.Trace("gg_sphere_jk")
    pairs, res = A.patch_pairs(tr)
    npatch = int(tr.final["patch"].max()) + 1
    v = J.design_matrix(res, pairs, npatch, gg=True, cpw="simple")
    cov = J.cov_jackknife(v)
    ref = tr.final["cov"]
    assert np.abs(cov - ref).max() <= 1e-10 * np.abs(ref).max()
    w = res[:, 0].sum(axis=0)
    np.testing.assert_allclose(A.finalize_xi(res[:, 3].sum(axis=0), w), tr.final["xip"],
                               rtol=1e-10, atol=1e-14)


def _ggg_sas_inputs(tr):
    call = [e for e in tr.events if e["op"] == "call" and e["method"] == "processAuto"][-1]
    new = [e for e in tr.events if e["op"] == "new" and e["cls"] == "GGGCorr"][0]
    nbins, min_sep, bin_size, max_n = new["args"][3], new["args"][1], new["args"][4], new["args"][9]
    return call, nbins, max_n, min_sep, bin_size


def test_tosas_restatement_matches_reference_python():
    """The oracle's restatement of the multipole finalisation and toSAS
    (treecorr/corr3base.py:2312-2396, 2489-2676), applied to the reference module's logged
    GGG outputs, gives the LogSAS result TreeCorr's own Python computed."""
    from oracle import tosas_oracle as O
    tr = A.Trace("ggg_mp")
    call, nbins, max_n, min_sep, bin_size = _ggg_sas_inputs(tr)
    outs = [tr.arr(r) for r in call["outs"]]
    w, gams = O.ggg_multipole_to_sas(outs, nbins, max_n, min_sep, bin_size,
                                     tr.final["sas_phi"])
    ref_w = tr.final["sas_weight"]
    assert np.abs(w - ref_w).max() <= 1e-12 * np.abs(ref_w).max()
    for k in range(4):
        ref = tr.final["sas_gam%d" % k]
        assert np.abs(gams[k] - ref).max() <= 1e-10 * np.abs(ref).max(), k
