"""Golden cases with the benchmark configurations' own shapes and binnings.

The catalogs are generated bit-identically on every machine (tests/golden/portable.py), so
the fixtures store only the reference's outputs plus a SHA-256 of the regenerated inputs,
which a test checks before it compares anything.

  gg_cfg1_bs1 / gg_cfg1_bs0   flat GG, 200,000 points U[0,1000']^2, 20 Log bins 1-100',
                              bin_slop 1 and 0, angle_slop 0.1 (the CPU-runnable config)
  gg_cfg2_bs01 / gg_cfg2_bs0  curved-sky GG, a 200,000-point sample of the 1000 deg^2 cap,
                              Arc, 30 Log bins 1-300', bin_slop 0.1 and 0, angle_slop 0.1
  gg_cfg1_exact / gg_cfg2_exact  the same catalogs and binnings with bin_slop 0 and
                              angle_slop 0 (every pair at its own separation)
  ggg_cfg4                    flat GGG LogMultipole, 4,000 points U[0,100']^2, 20 Log bins
                              1-50', max_n 30, the reference's default bin_slop / angle_slop
                              (NC = 4 nbins = 80 columns in the tensor-core contraction)
"""
import hashlib

import numpy as np

import portable

ARCMIN = np.pi / 180. / 60.

# name: (dtype, coords, metric, catalog, min_sep, max_sep, nbins, bin_slop, angle_slop)
BENCH2 = {
    "gg_cfg1_bs1": ("G", "flat", "Euclidean", "cfg1", 1., 100., 20, 1.0, 0.1),
    "gg_cfg1_bs0": ("G", "flat", "Euclidean", "cfg1", 1., 100., 20, 0.0, 0.1),
    "gg_cfg2_bs01": ("G", "spherical", "Arc", "cfg2", 1. * ARCMIN, 300. * ARCMIN, 30, 0.1, 0.1),
    "gg_cfg2_bs0": ("G", "spherical", "Arc", "cfg2", 1. * ARCMIN, 300. * ARCMIN, 30, 0.0, 0.1),
    # bin_slop 0 and angle_slop 0: every pair in range is counted at its own separation (the
    # accuracy the benchmark metric asks for); the GPU evaluates these in leaf-pair tiles.
    "gg_cfg1_exact": ("G", "flat", "Euclidean", "cfg1", 1., 100., 20, 0.0, 0.0),
    "gg_cfg2_exact": ("G", "spherical", "Arc", "cfg2", 1. * ARCMIN, 300. * ARCMIN, 30, 0.0, 0.0),
}

# name: (n, side, min_sep, max_sep, nbins, max_n)
BENCH3 = {
    "ggg_cfg4": (4000, 100., 1., 50., 20, 30),
}

CATALOGS = {
    "cfg1": lambda: portable.flat_catalog(20260101, 200_000, 1000.0, sigma=0.2),
    "cfg2": lambda: portable.cap_catalog(20260102, 200_000, portable.COS_R_1000DEG2, sigma=0.25),
}


def catalog_hash(cat):
    h = hashlib.sha256()
    for k in ("x", "y", "z", "g1", "g2", "k", "w"):
        v = cat.get(k)
        if v is not None:
            h.update(k.encode())
            h.update(np.ascontiguousarray(v, dtype=np.float64).tobytes())
    return h.hexdigest()


def bench2_inputs(name):
    return CATALOGS[BENCH2[name][3]]()


def bench2_spec(name):
    dtype, coords, metric, catname, lo, hi, nb, bs, asl = BENCH2[name]
    bin_size = np.log(hi / lo) / nb
    b = bs * bin_size
    if metric == "Euclidean":
        b1 = min(asl, b)
        min_size, max_size = lo * b1 / (2 + 3 * b1), hi * b1
    else:
        min_size, max_size = 0.0, 0.0
    bins = dict(min_sep=lo, max_sep=hi, nbins=nb, bin_size=bin_size, b=b, a=asl)
    return dict(dtype=dtype, coords=coords, metric=metric, bins=bins, min_size=min_size,
                max_size=max_size, split="mean", brute=False, min_top=3, max_top=10)


def bench3_inputs(name):
    n, side = BENCH3[name][:2]
    return portable.flat_catalog(20260104, n, side, sigma=0.25)


def bench3_spec(name):
    """The reference's LogMultipole defaults (treecorr/corr3base.py:714-726): angle_slop =
    pi/(2 max_n + 1); bin_slop = 1 if bin_size <= 0.1 else 0.1 / bin_size."""
    n, side, lo, hi, nb, max_n = BENCH3[name]
    bin_size = np.log(hi / lo) / nb
    bs = 1.0 if bin_size <= 0.1 else 0.1 / bin_size
    b = bs * bin_size
    a = np.pi / (2 * max_n + 1)
    b1 = min(a, b)
    min_size, max_size = 2 * lo * b1 / (2. + 3 * b1), hi * b1
    return dict(coords="flat", metric="Euclidean", n=n, min_sep=lo, max_sep=hi, nbins=nb,
                max_n=max_n, bin_size=bin_size, b=b, a=a, min_size=min_size,
                max_size=max_size)
