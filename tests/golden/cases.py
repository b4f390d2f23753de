"""Seeded synthetic cases shared by the golden-fixture generator and the tests.

Each case is a small catalog (seconds for the oracle) plus the binning/slop arguments that
the reference's Python layer would pass to its native module.  Distributions follow the
benchmark configurations at reduced size: flat U[0,L]^2 positions, Gaussian shears clipped
to |g|<0.9, weights U[0.5,1.5]; curved-sky points uniform in a small cap.
"""
import numpy as np


def flat_catalog(rng, n, L=100.0, clumped=False):
    if clumped:
        nc = max(n // 50, 1)
        cen = rng.uniform(0, L, size=(nc, 2))
        k = rng.integers(0, nc, size=n)
        xy = cen[k] + rng.normal(0, L / 50., size=(n, 2))
        x, y = xy[:, 0].copy(), xy[:, 1].copy()   # contiguous, like Catalog's arrays
    else:
        x = rng.uniform(0, L, n)
        y = rng.uniform(0, L, n)
    g1 = rng.normal(0, 0.2, n)
    g2 = rng.normal(0, 0.2, n)
    gabs = np.hypot(g1, g2)
    shrink = np.where(gabs > 0.9, 0.9 / gabs, 1.0)
    g1 *= shrink
    g2 *= shrink
    k = rng.normal(0, 0.02, n)
    w = rng.uniform(0.5, 1.5, n)
    return dict(x=x, y=y, z=None, g1=g1, g2=g2, k=k, w=w)


def sphere_catalog(rng, n, radius_deg=5.0, ra0=30.0, dec0=-20.0):
    """Uniform in a spherical cap; returns unit vectors like Catalog._generate_xyz
    (treecorr/catalog.py:1609-1622: x=cos(dec)cos(ra), y=cos(dec)sin(ra), z=sin(dec))."""
    cosr = np.cos(np.radians(radius_deg))
    u = rng.uniform(cosr, 1.0, n)
    phi = rng.uniform(0, 2 * np.pi, n)
    s = np.sqrt(1 - u * u)
    # cap around the pole, then rotate to (ra0, dec0)
    v = np.stack([s * np.cos(phi), s * np.sin(phi), u])
    th = np.radians(90.0 - dec0)
    Ry = np.array([[np.cos(th), 0, np.sin(th)], [0, 1, 0], [-np.sin(th), 0, np.cos(th)]])
    a = np.radians(ra0)
    Rz = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    v = Rz @ Ry @ v
    g1 = rng.normal(0, 0.25, n)
    g2 = rng.normal(0, 0.25, n)
    k = rng.normal(0, 0.02, n)
    w = rng.uniform(0.5, 1.5, n)
    return dict(x=v[0].copy(), y=v[1].copy(), z=v[2].copy(), g1=g1, g2=g2, k=k, w=w)


def threed_catalog(rng, n, L=100.0):
    x = rng.uniform(0, L, n)
    y = rng.uniform(0, L, n)
    z = rng.uniform(200, 200 + L, n)
    g1 = rng.normal(0, 0.2, n)
    g2 = rng.normal(0, 0.2, n)
    k = rng.normal(0, 0.02, n)
    w = rng.uniform(0.5, 1.5, n)
    return dict(x=x, y=y, z=z, g1=g1, g2=g2, k=k, w=w)


ARCMIN = np.pi / 180. / 60.

# name: (dtype, coords, metric, generator, n, n2 (cross) or 0, min_sep, max_sep, nbins,
#        bin_slop, angle_slop, split, brute, min_top, max_top)
CASES = {
    "gg_flat_bs1":      ("G", "flat", "Euclidean", "flat", 3000, 0, 1., 20., 10, 1.0, 0.1, "mean", False, 3, 10),
    "gg_flat_bs0":      ("G", "flat", "Euclidean", "flat", 3000, 0, 1., 20., 10, 0.0, 0.1, "mean", False, 3, 10),
    "gg_flat_exact":    ("G", "flat", "Euclidean", "flat", 1500, 0, 1., 20., 10, 0.0, 0.0, "mean", False, 3, 10),
    "gg_flat_brute":    ("G", "flat", "Euclidean", "flat", 800, 0, 1., 20., 10, 1.0, 0.1, "mean", True, 3, 10),
    "gg_flat_clumped":  ("G", "flat", "Euclidean", "clumped", 6000, 0, 0.5, 30., 15, 1.0, 0.1, "mean", False, 3, 10),
    "gg_flat_middle":   ("G", "flat", "Euclidean", "flat", 3000, 0, 1., 20., 10, 1.0, 0.1, "middle", False, 3, 10),
    "gg_flat_median":   ("G", "flat", "Euclidean", "flat", 3000, 0, 1., 20., 10, 1.0, 0.1, "median", False, 3, 10),
    "gg_flat_cross":    ("G", "flat", "Euclidean", "flat", 2000, 1500, 1., 20., 10, 0.5, 0.1, "mean", False, 3, 10),
    "nn_flat_bs1":      ("N", "flat", "Euclidean", "flat", 4000, 0, 1., 25., 12, 1.0, 0.1, "mean", False, 3, 10),
    "nn_flat_cross":    ("N", "flat", "Euclidean", "flat", 2500, 3000, 1., 25., 12, 0.0, 0.1, "mean", False, 3, 10),
    "kk_flat_bs1":      ("K", "flat", "Euclidean", "flat", 3000, 0, 1., 20., 10, 1.0, 1.0, "mean", False, 3, 10),
    "kk_flat_bs0":      ("K", "flat", "Euclidean", "flat", 3000, 0, 1., 20., 10, 0.0, 1.0, "mean", False, 3, 10),
    "gg_sphere_arc":    ("G", "spherical", "Arc", "sphere", 3000, 0, 2. * ARCMIN, 60. * ARCMIN, 10, 0.5, 0.1, "mean", False, 3, 10),
    "gg_sphere_arc_bs0": ("G", "spherical", "Arc", "sphere", 2000, 0, 2. * ARCMIN, 60. * ARCMIN, 10, 0.0, 0.1, "mean", False, 3, 10),
    "gg_sphere_euc":    ("G", "spherical", "Euclidean", "sphere", 3000, 0, 2. * ARCMIN, 60. * ARCMIN, 10, 1.0, 0.1, "mean", False, 3, 10),
    "nn_sphere_arc_cross": ("N", "spherical", "Arc", "sphere", 2000, 2500, 2. * ARCMIN, 60. * ARCMIN, 10, 0.1, 0.1, "mean", False, 3, 10),
    "kk_sphere_arc":    ("K", "spherical", "Arc", "sphere", 3000, 0, 2. * ARCMIN, 60. * ARCMIN, 10, 1.0, 1.0, "mean", False, 3, 10),
    "gg_3d":            ("G", "3d", "Euclidean", "threed", 3000, 0, 1., 30., 10, 1.0, 0.1, "mean", False, 3, 10),
    "nn_3d":            ("N", "3d", "Euclidean", "threed", 3000, 0, 1., 30., 10, 0.5, 0.1, "mean", False, 3, 10),
    # The other 2-point classes (src/Corr2.cpp:1204-1232): a two-letter dtype is (d1, d2) of
    # a cross correlation; Z, V, T, Q fields take the complex columns (g1, g2).
    "nk_flat_cross":    ("NK", "flat", "Euclidean", "flat", 2000, 2500, 1., 20., 10, 1.0, 0.1, "mean", False, 3, 10),
    "ng_flat_cross":    ("NG", "flat", "Euclidean", "flat", 2500, 3000, 1., 20., 10, 0.5, 0.1, "mean", False, 3, 10),
    "kg_sphere_cross":  ("KG", "spherical", "Arc", "sphere", 2000, 2500, 2. * ARCMIN, 60. * ARCMIN, 10, 0.5, 0.1, "mean", False, 3, 10),
    "ng_sphere_bs0":    ("NG", "spherical", "Arc", "sphere", 1200, 1500, 2. * ARCMIN, 60. * ARCMIN, 8, 0.0, 0.1, "mean", False, 3, 10),
    "nz_flat_cross":    ("NZ", "flat", "Euclidean", "flat", 2000, 2500, 1., 20., 10, 1.0, 0.1, "mean", False, 3, 10),
    "kv_sphere_cross":  ("KV", "spherical", "Arc", "sphere", 2000, 2500, 2. * ARCMIN, 60. * ARCMIN, 10, 0.5, 0.1, "mean", False, 3, 10),
    "nt_3d_cross":      ("NT", "3d", "Euclidean", "threed", 2000, 2500, 1., 30., 10, 1.0, 0.1, "mean", False, 3, 10),
    "kq_flat_cross":    ("KQ", "flat", "Euclidean", "flat", 2000, 2500, 1., 20., 10, 1.0, 0.1, "mean", False, 3, 10),
    "zz_sphere":        ("Z", "spherical", "Arc", "sphere", 2500, 0, 2. * ARCMIN, 60. * ARCMIN, 10, 0.5, 0.1, "mean", False, 3, 10),
    "vv_flat":          ("V", "flat", "Euclidean", "flat", 2500, 0, 1., 20., 10, 1.0, 0.1, "mean", False, 3, 10),
    "vv_sphere":        ("V", "spherical", "Arc", "sphere", 2500, 0, 2. * ARCMIN, 60. * ARCMIN, 10, 0.5, 0.1, "mean", False, 3, 10),
    "tt_sphere":        ("T", "spherical", "Arc", "sphere", 2500, 0, 2. * ARCMIN, 60. * ARCMIN, 10, 0.5, 0.1, "mean", False, 3, 10),
    "qq_flat":          ("Q", "flat", "Euclidean", "flat", 2500, 0, 1., 20., 10, 1.0, 0.1, "mean", False, 3, 10),
    "qq_3d":            ("Q", "3d", "Euclidean", "threed", 2500, 0, 1., 30., 10, 1.0, 0.1, "mean", False, 3, 10),
    "tt_flat_cross":    ("T", "flat", "Euclidean", "flat", 2000, 2500, 1., 20., 10, 0.5, 0.1, "mean", False, 3, 10),
    # Exact mode (angle_slop 0, or brute fields): every accepted pair is a pair of leaves,
    # which the GPU evaluates in leaf-pair tiles.
    "gg_sphere_exact":  ("G", "spherical", "Arc", "sphere", 2500, 0, 2. * ARCMIN, 60. * ARCMIN, 10, 0.0, 0.0, "mean", False, 3, 10),
    "nn_flat_exact_cross": ("N", "flat", "Euclidean", "flat", 2000, 2500, 1., 20., 10, 0.0, 0.0, "mean", False, 3, 10),
    "kk_sphere_exact":  ("K", "spherical", "Arc", "sphere", 2500, 0, 2. * ARCMIN, 60. * ARCMIN, 10, 0.5, 0.0, "mean", False, 3, 10),
    "ng_3d_exact_cross": ("NG", "3d", "Euclidean", "threed", 1500, 2000, 1., 30., 10, 0.0, 0.0, "mean", False, 3, 10),
    "tt_sphere_exact_median": ("T", "spherical", "Arc", "sphere", 2000, 0, 2. * ARCMIN, 60. * ARCMIN, 10, 0.0, 0.0, "median", False, 3, 10),
    "kg_flat_exact_clumped": ("KG", "flat", "Euclidean", "clumped", 2500, 2500, 0.5, 30., 15, 0.0, 0.0, "mean", False, 3, 10),
    "qq_flat_brute":    ("Q", "flat", "Euclidean", "flat", 1200, 0, 1., 20., 10, 1.0, 0.1, "mean", True, 3, 10),
    "zz_sphere_brute_euc": ("Z", "spherical", "Euclidean", "sphere", 1500, 0, 2. * ARCMIN, 60. * ARCMIN, 10, 0.5, 0.1, "mean", True, 3, 10),
}


def kinds(dtype):
    """(d1, d2) data kinds of a case's dtype ("G" -> ("G", "G"), "NG" -> ("N", "G"))."""
    return dtype[0], dtype[-1]


def xi_count(dtype):
    """Number of xi arrays the reference's Corr2<D1,D2> fills (XiData, include/Corr2.h)."""
    d1, d2 = kinds(dtype)
    if d1 == "N" and d2 == "N":
        return 0
    if d2 in "NK":
        return 1
    if d1 in "NK":
        return 2
    return 4


def make_inputs(name, seed=8675309):
    spec = CASES[name]
    gen, n, n2 = spec[3], spec[4], spec[5]
    rng = np.random.default_rng(seed + sum(map(ord, name)))
    f = {"flat": lambda r, m: flat_catalog(r, m),
         "clumped": lambda r, m: flat_catalog(r, m, clumped=True),
         "sphere": lambda r, m: sphere_catalog(r, m),
         "threed": lambda r, m: threed_catalog(r, m)}[gen]
    cat1 = f(rng, n)
    cat2 = f(rng, n2) if n2 else None
    return cat1, cat2


def spec_dict(name):
    (dtype, coords, metric, gen, n, n2, min_sep, max_sep, nbins, bin_slop, angle_slop,
     split, brute, min_top, max_top) = CASES[name]
    return dict(dtype=dtype, coords=coords, metric=metric, n=n, n2=n2, min_sep=min_sep,
                max_sep=max_sep, nbins=nbins, bin_slop=bin_slop, angle_slop=angle_slop,
                split=split, brute=brute, min_top=min_top, max_top=max_top)
