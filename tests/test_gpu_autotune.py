"""GPU tests of the autotuner (tile leaf size and expansion queue depth; no reference
counterpart): it picks values from its candidate sets, leaves the output arrays untouched,
caches its choice per configuration, and the tuned correlation still equals the reference's
output (tuning never changes a result)."""
import os
import sys

import numpy as np
import pytest

import helpers as H
from cases_bench import bench2_inputs, bench2_spec

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _corr(T, bins, out):
    return T.GGCorr(T.Log, bins["min_sep"], bins["max_sep"], bins["nbins"], bins["bin_size"],
                    bins["b"], bins["a"], -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
                    out["xi0"], out["xi1"], out["xi2"], out["xi3"], out["meanr"],
                    out["meanlogr"], out["weight"], out["npairs"])


@pytest.mark.parametrize("name", ["gg_cfg2_exact", "gg_cfg2_bs01"])
def test_autotune_keeps_results(gpu_lib, name):
    T = gpu_lib
    s = bench2_spec(name)
    g = np.load(os.path.join(HERE, name + ".npz"))
    cat = bench2_inputs(name)
    f = H.gpu_field(T, "G", s["coords"], cat, s["min_size"], s["max_size"])
    out = {k: np.zeros(s["bins"]["nbins"]) for k in H.OUT_KEYS}
    c = _corr(T, s["bins"], out)
    tune = c.autotune(f, metric=T.Arc, frac=0.1)
    print(name, tune)
    assert not any(out[k].any() for k in H.OUT_KEYS)     # the samples add nothing
    exact = s["bins"]["a"] == 0.
    if exact:
        assert tune["tile_leaf"] in (24, 32, 40, 48, 56, 64)
        assert tune["ms"] > 0.
    else:
        assert tune["tile_leaf"] == 0
    assert tune["chunk"] == 0 or (tune["chunk"] & (tune["chunk"] - 1)) == 0
    c.processAuto(f, False, False, T.Arc)
    ref = {k: g["ref_" + k] for k in H.OUT_KEYS}
    H.assert_outputs_close(out, ref, "G", rtol=1e-5, label=name + " tuned")
    # A second corr with the same configuration takes the cached choice at once.
    out2 = {k: np.zeros(s["bins"]["nbins"]) for k in H.OUT_KEYS}
    c2 = _corr(T, s["bins"], out2)
    tune2 = c2.autotune(f, metric=T.Arc, frac=0.1)
    assert tune2["tile_leaf"] == tune["tile_leaf"] and tune2["chunk"] == tune["chunk"]
    assert tune2["ms"] == 0.


def test_tuning_values_checked_and_inert(gpu_lib):
    """Explicit tuning values: out-of-range ones are refused; in-range ones give the same
    result as the defaults."""
    T = gpu_lib
    s, c1, c2, bins, min_size, max_size, ref = H.load_case("gg_sphere_exact")
    f = H.gpu_field(T, "G", "spherical", c1, min_size, max_size)
    out = {k: np.zeros(bins["nbins"]) for k in H.OUT_KEYS}
    c = _corr(T, bins, out)
    with pytest.raises(ValueError):
        c.setTuning(tile_leaf=65)
    with pytest.raises(ValueError):
        c.setTuning(chunk=100)
    for leaf, chunk in ((8, 1 << 16), (64, 0), (24, 1 << 20)):
        for k in out:
            out[k][:] = 0.
        c.setTuning(tile_leaf=leaf, chunk=chunk)
        c.processAuto(f, False, False, T.Arc)
        H.assert_outputs_close(out, ref, "G", rtol=1e-5, label=f"leaf {leaf} chunk {chunk}")
