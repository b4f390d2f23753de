"""Seeded k-means cases shared by the golden-fixture generator and the tests.

Each case is a small catalog, the patch count and the top-level recursion limits of the
N field that treecorr/catalog.py builds for k-means (max_top = bit_length(npatch) - 1,
min_size 0, max_size inf, split 'mean').  The cases cover both branches of
InitializeCentersTree (more top cells than centres: Floyd's and Fisher-Yates selection;
fewer: the recursive split) and all three geometries.
"""
import numpy as np

from cases import flat_catalog, sphere_catalog, threed_catalog

# name: (generator, n, npatch, min_top, max_top, coords)
KM_CASES = {
    "km_flat":      ("flat", 4000, 20, 3, 4, "flat"),
    "km_flat_floyd": ("flat", 3000, 10, 5, 5, "flat"),
    "km_clumped":   ("clumped", 5000, 40, 3, 5, "flat"),
    "km_sphere":    ("sphere", 5000, 30, 3, 4, "spherical"),
    "km_3d":        ("threed", 3000, 16, 5, 5, "3d"),
}

KM_SEED = 12345       # the seed passed to the initialisations
KM_TOL = 1.e-5
KM_MAX_ITER = 200


def km_inputs(name, seed=4242):
    gen, n = KM_CASES[name][0], KM_CASES[name][1]
    rng = np.random.default_rng(seed + sum(map(ord, name)))
    f = {"flat": lambda r, m: flat_catalog(r, m),
         "clumped": lambda r, m: flat_catalog(r, m, clumped=True),
         "sphere": lambda r, m: sphere_catalog(r, m),
         "threed": lambda r, m: threed_catalog(r, m)}[gen]
    return f(rng, n)


def km_spec(name):
    gen, n, npatch, min_top, max_top, coords = KM_CASES[name]
    return dict(gen=gen, n=n, npatch=npatch, min_top=min_top, max_top=max_top, coords=coords)
