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
