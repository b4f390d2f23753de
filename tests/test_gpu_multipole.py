"""GPU parity of the GGG LogMultipole accumulation against the reference's golden outputs
and the oracle."""
import os
import sys

import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu

MP_OUT = ("gam0r", "gam0i", "gam1r", "gam1i", "gam2r", "gam2i", "gam3r", "gam3i",
          "meand1", "meanlogd1", "meand2", "meanlogd2", "meand3", "meanlogd3", "meanu",
          "meanv", "weight", "weight_im", "ntri")


def gpu_multipole(T, s, cat, min_size, max_size):
    nb, mn = s["nbins"], s["max_n"]
    shape = (nb, nb, 2 * mn + 1)
    out = {k: np.zeros(shape) for k in MP_OUT}
    corr = T.GGGCorr(T.LogMultipole, s["min_sep"], s["max_sep"], nb, s["bin_size"], s["b"],
                     s["a"], 0., 0., mn, 0., 0., 0., 0., 0, 0., 0.,
                     -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
                     *[out[k] for k in MP_OUT])
    f = H.gpu_field(T, "G", s["coords"], cat, min_size, max_size)
    m = T.Euclidean if s["metric"] == "Euclidean" else T.Arc
    corr.processAuto(f, False, False, m)
    return out


@pytest.mark.parametrize("name", ["ggg_flat_mp", "ggg_flat_mp_n20", "ggg_flat_mp_bs0",
                                  "ggg_sphere_mp"])
def test_multipole_golden(gpu_lib, name):
    from cases3 import spec3
    s = spec3(name)
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    cat = {k[3:]: g[k] for k in g.files if k.startswith("c1_")}
    out = gpu_multipole(gpu_lib, s, cat, float(g["min_size"]), float(g["max_size"]))
    assert np.array_equal(out["ntri"], g["ref_ntri"]), name
    for k in MP_OUT:
        r = g["ref_" + k]
        scale = max(np.abs(r).max(), 1e-300)
        err = np.abs(out[k] - r).max() / scale
        # FP64 throughout; only the order of some sums differs from the reference.
        assert err <= 1e-10, f"{name} {k}: {err:.3e}"
