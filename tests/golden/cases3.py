"""Seeded cases for the GGG LogMultipole (3-point) golden fixtures."""
import numpy as np

from cases import flat_catalog, sphere_catalog, ARCMIN

# name: (coords, metric, generator, n, min_sep, max_sep, nbins, max_n, bin_slop, angle_slop)
# angle_slop None -> the reference default pi/(2*max_n+1) (treecorr/corr3base.py:714-716);
# bin_slop None -> its default (1 if bin_size <= 0.1 else 0.1/bin_size, 719-726).
CASES3 = {
    "ggg_flat_mp":      ("flat", "Euclidean", "flat", 800, 2., 20., 5, 10, None, None),
    "ggg_flat_mp_n20":  ("flat", "Euclidean", "flat", 600, 1., 30., 8, 20, None, None),
    "ggg_flat_mp_bs0":  ("flat", "Euclidean", "flat", 300, 2., 20., 5, 6, 0.0, 0.0),
    "ggg_sphere_mp":    ("spherical", "Arc", "sphere", 700, 4. * ARCMIN, 40. * ARCMIN, 5, 8, None, None),
}


def make_inputs3(name, seed=20240601):
    spec = CASES3[name]
    gen, n = spec[2], spec[3]
    rng = np.random.default_rng(seed + sum(map(ord, name)))
    if gen == "flat":
        return flat_catalog(rng, n, L=60.)
    return sphere_catalog(rng, n, radius_deg=1.0)


def spec3(name):
    coords, metric, gen, n, lo, hi, nb, max_n, bs, asl = CASES3[name]
    bin_size = np.log(hi / lo) / nb
    if bs is None:
        bs = 1.0 if bin_size <= 0.1 else 0.1 / bin_size
    b = bs * bin_size
    a = np.pi / (2 * max_n + 1) if asl is None else asl
    return dict(coords=coords, metric=metric, n=n, min_sep=lo, max_sep=hi, nbins=nb,
                max_n=max_n, bin_size=bin_size, b=b, a=a)
