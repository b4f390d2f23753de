"""GenerateXYZ (src/KMeans.cpp:1013-1050) against the reference's own outputs
(tests/golden/generate_xyz.npz, made by tests/golden/make_golden.py --xyz)."""
import os

import numpy as np
import pytest

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "generate_xyz.npz"))


def restated(ra, dec, r=None):
    """The oracle: the reference's formulas in numpy."""
    x, y, z = np.cos(dec) * np.cos(ra), np.cos(dec) * np.sin(ra), np.sin(dec)
    if r is not None:
        x, y, z = x * r, y * r, z * r
    return x, y, z


def test_oracle_matches_reference():
    for tag, r in (("", None), ("_r", G["r"])):
        got = restated(G["ra"], G["dec"], r)
        for a, k in zip(got, "xyz"):
            ref = G[k + tag]
            assert np.allclose(a, ref, rtol=4e-16, atol=4e-16 * np.abs(ref).max())


@pytest.mark.gpu
def test_gpu_matches_reference(gpu_lib):
    T = gpu_lib
    n = len(G["ra"])
    for tag, r in (("", np.array([])), ("_r", G["r"])):
        x, y, z = np.zeros(n), np.zeros(n), np.zeros(n)
        T.GenerateXYZ(x, y, z, G["ra"], G["dec"], r)
        for a, k in zip((x, y, z), "xyz"):
            ref = G[k + tag]
            # CUDA's sincos and libm's differ by at most an ulp or two.
            assert np.abs(a - ref).max() <= 4e-16 * np.abs(ref).max(), (k, tag)
