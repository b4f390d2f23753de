"""Properties of the 2-point path at the benchmark's full size (10M points on a 1000 deg^2
cap, Arc, 30 Log bins 1-300', bin_slop 0.1), where no oracle finishes in seconds:

* npairs depends only on the positions: NN, KK and GG give the same integer counts;
* the correlations are bilinear in the data: doubling g (k) multiplies xi by 4, with the
  same weights and counts.
"""
import sys

import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu

ARCMIN = np.pi / 180. / 60.
N = 10_000_000


def cap_catalog(n, seed=99, area_deg2=1000.0):
    rng = np.random.default_rng(seed)
    r = np.arccos(1 - area_deg2 * (np.pi / 180) ** 2 / (2 * np.pi))
    u = rng.uniform(np.cos(r), 1.0, n)
    phi = rng.uniform(0, 2 * np.pi, n)
    s = np.sqrt(1 - u * u)
    x, y, z = s * np.cos(phi), s * np.sin(phi), u
    # rotate the cap from the pole to dec = -30 deg
    a = np.radians(120.0)
    x, z = x * np.cos(a) + z * np.sin(a), -x * np.sin(a) + z * np.cos(a)
    return dict(x=np.ascontiguousarray(x), y=np.ascontiguousarray(y),
                z=np.ascontiguousarray(z), g1=rng.normal(0, 0.25, n),
                g2=rng.normal(0, 0.25, n), k=rng.normal(0, 0.02, n),
                w=rng.uniform(0.5, 1.5, n))


def test_full_size_counts_and_bilinearity(gpu_lib):
    T = gpu_lib
    cat = cap_catalog(N)
    nb = 30
    lo, hi = 1.0 * ARCMIN, 300.0 * ARCMIN
    bsz = np.log(hi / lo) / nb
    bins = dict(min_sep=lo, max_sep=hi, nbins=nb, bin_size=bsz, b=0.1 * bsz, a=0.1)
    run = {}
    for tag, dt, scale in (("gg", "G", 1.0), ("gg2", "G", 2.0), ("kk", "K", 1.0),
                           ("kk2", "K", 2.0), ("nn", "N", 1.0)):
        c = dict(cat)
        c["g1"], c["g2"], c["k"] = cat["g1"] * scale, cat["g2"] * scale, cat["k"] * scale
        f = H.gpu_field(T, dt, "spherical", c, 0.0, 0.0)
        run[tag] = H.gpu_process(T, dt, "Arc", bins, f)
        del f
    npairs = run["nn"]["npairs"]
    assert npairs.sum() > 1e12
    for tag in ("gg", "gg2", "kk", "kk2"):
        assert np.array_equal(run[tag]["npairs"], npairs), tag
    wmax = np.abs(run["nn"]["weight"]).max()
    for tag in ("gg", "gg2", "kk", "kk2"):
        np.testing.assert_allclose(run[tag]["weight"], run["nn"]["weight"], rtol=0,
                                   atol=1e-8 * wmax, err_msg=tag)
    # Doubling a float payload is exact, so xi scales by 4 up to the run-to-run order of
    # the FP32 partial sums; judged against the bin's scale (at least 1e-6 of the weight).
    for base, two, keys in (("gg", "gg2", ("xi0", "xi1", "xi2", "xi3")), ("kk", "kk2", ("xi0",))):
        for k in keys:
            a, b = run[base][k], run[two][k]
            scale = max(np.abs(a).max(), 1e-6 * wmax)
            assert np.abs(b - 4.0 * a).max() <= 4e-5 * scale, (base, k)
