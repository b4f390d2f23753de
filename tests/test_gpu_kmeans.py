"""k-means patches on the GPU (KMeansInit*, KMeansRun, KMeansAssign, QuickAssign,
SelectPatch) against the reference's own outputs (tests/golden/km_*.npz) and the oracle."""
import os

import numpy as np
import pytest

from cases import flat_catalog, sphere_catalog
from cases_km import KM_CASES, KM_MAX_ITER, KM_SEED, KM_TOL, km_spec
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
COORDS = {"flat": "Flat", "spherical": "Sphere", "3d": "ThreeD"}


def load(name):
    d = np.load(os.path.join(GOLD, name + ".npz"))
    return {k: d[k] for k in d.files}


def gpu_nfield(T, coords, x, y, z, w, min_top, max_top):
    cls = getattr(T, "NField" + COORDS[coords])
    empty = np.array([])
    return cls(x, y, z if z is not None else empty, w, empty, 0.0, np.inf, T.SplitMethod.Mean,
               0, False, min_top, max_top)


def oracle_nfield(coords, x, y, z, w, min_top, max_top):
    return O.OracleField("N", coords, x, y, z, w=w, min_size=0.0, max_size=np.inf,
                         split_method="mean", min_top=min_top, max_top=max_top)


def close_centres(a, b, msg=""):
    np.testing.assert_allclose(a, b, rtol=0, atol=1e-14 * max(1.0, np.abs(b).max()), err_msg=msg)


def case_fields(T, name):
    g = load(name)
    s = km_spec(name)
    args = (s["coords"], g["x"], g["y"], g.get("z"), g["w"], s["min_top"], s["max_top"])
    return g, s, gpu_nfield(T, *args), oracle_nfield(*args)


@pytest.mark.parametrize("name", sorted(KM_CASES))
def test_init_matches_reference_and_oracle(gpu_lib, name):
    g, s, f, of = case_fields(gpu_lib, name)
    npatch = s["npatch"]
    dim = 2 if s["coords"] == "flat" else 3
    for tag, meth, init in (("tree", f.KMeansInitTree, "tree"),
                            ("rand", f.KMeansInitRand, "random"),
                            ("kmpp", f.KMeansInitKMPP, "kmeans++")):
        c = np.zeros((npatch, dim))
        meth(c, npatch, KM_SEED)
        # Same draws, same cells; cell centroids summed in another order by the device
        # build (and ~0.6% of the reference's sphere points normalised by a reciprocal
        # multiply under -ffast-math): agreement to a few ulp of the coordinates.
        close_centres(c, of.kmeans_init(npatch, init, KM_SEED), tag)
        close_centres(c, g["init_" + tag], tag)


@pytest.mark.parametrize("name", sorted(KM_CASES))
def test_run_matches_reference(gpu_lib, name):
    g, s, f, of = case_fields(gpu_lib, name)
    npatch = s["npatch"]
    for tag, iters, alt in (("it1", 1, False), ("it3", 3, False), ("run", KM_MAX_ITER, False),
                            ("alt_it1", 1, True), ("alt_it3", 3, True),
                            ("alt_run", KM_MAX_ITER, True)):
        c = g["init_tree"].copy()
        f.KMeansRun(c, npatch, iters, KM_TOL, alt)
        # Cell sums in another order than the reference's recursion: rounding only.
        scale = np.abs(g[tag]).max()
        np.testing.assert_allclose(c, g[tag], rtol=0, atol=1e-12 * scale, err_msg=tag)
        oc, oit = of.kmeans_run(g["init_tree"], iters, KM_TOL, alt)
        assert f.kmeans_iterations() == oit, tag
    for tag, cen in (("assign", "run"), ("alt_assign", "alt_run")):
        pat = np.zeros(s["n"], dtype=np.int64)
        f.KMeansAssign(g[cen], npatch, pat)
        assert np.array_equal(pat, g[tag]), tag


@pytest.mark.parametrize("name", sorted(KM_CASES))
def test_quick_assign_and_select_patch_match_reference(gpu_lib, name):
    T = gpu_lib
    g = load(name)
    npatch = km_spec(name)["npatch"]
    z = g["z"] if "z" in g else np.array([])
    q = np.zeros(len(g["x"]), dtype=np.int64)
    T.QuickAssign(g["run"], npatch, g["x"], g["y"], z, q)
    assert np.array_equal(q, g["quick"])
    for pp in (0, npatch - 1):
        use = np.zeros(len(g["x"]), dtype=np.int64)
        T.SelectPatch(pp, g["run"], npatch, g["x"], g["y"], z, use)
        assert np.array_equal(use, g["select_%d" % pp])


@pytest.mark.parametrize("geom", ["flat", "spherical"])
def test_larger_catalog_against_oracle(gpu_lib, geom):
    """200K points, 64 patches: the GPU run tracks the oracle, and the tree assignment of
    the plain criterion equals the point-wise nearest centre (QuickAssign)."""
    T = gpu_lib
    rng = np.random.default_rng(31 if geom == "flat" else 32)
    n, npatch = 200_000, 64
    if geom == "flat":
        cat = flat_catalog(rng, n, L=1000.)
    else:
        cat = sphere_catalog(rng, n, radius_deg=10.)
    args = (geom, cat["x"], cat["y"], cat["z"], cat["w"], 3, int(npatch).bit_length() - 1)
    f, of = gpu_nfield(T, *args), oracle_nfield(*args)
    dim = 2 if geom == "flat" else 3
    c0 = np.zeros((npatch, dim))
    f.KMeansInitTree(c0, npatch, 777)
    close_centres(c0, of.kmeans_init(npatch, "tree", 777))
    c = c0.copy()
    f.KMeansRun(c, npatch, 30, 0., False)
    oc, _ = of.kmeans_run(c0, 30, 0., False)
    np.testing.assert_allclose(c, oc, rtol=0, atol=1e-11 * np.abs(oc).max())
    pat = np.zeros(n, dtype=np.int64)
    f.KMeansAssign(c, npatch, pat)
    q = np.zeros(n, dtype=np.int64)
    T.QuickAssign(c, npatch, cat["x"], cat["y"], cat["z"] if cat["z"] is not None else np.array([]), q)
    assert np.array_equal(pat, q)
    assert np.array_equal(pat, of.kmeans_assign(c))
    assert (np.bincount(pat, minlength=npatch) > 0).all()


def test_edge_cases(gpu_lib):
    T = gpu_lib
    rng = np.random.default_rng(3)
    cat = flat_catalog(rng, 500)
    f = gpu_nfield(T, "flat", cat["x"], cat["y"], None, cat["w"], 3, 10)
    of = oracle_nfield("flat", cat["x"], cat["y"], None, cat["w"], 3, 10)
    # One patch: every point in patch 0; the centre is the mean of the top cells' centroids
    # weighted by their float weights (UpdateCenters), ~1e-8 from the exact weighted mean.
    c = np.zeros((1, 2))
    f.KMeansInitTree(c, 1, 5)
    c0 = c.copy()
    f.KMeansRun(c, 1, 10, 1e-5, False)
    close_centres(c, of.kmeans_run(c0, 10, 1e-5, False)[0])
    w = cat["w"]
    np.testing.assert_allclose(c[0], [np.sum(w * cat["x"]) / w.sum(), np.sum(w * cat["y"]) / w.sum()],
                               rtol=1e-7)
    pat = np.full(500, 7, dtype=np.int64)
    f.KMeansAssign(c, 1, pat)
    assert (pat == 0).all()
    # max_iter = 0 leaves the centres alone.
    c2 = np.array([[10., 20.], [80., 70.]])
    c3 = c2.copy()
    f.KMeansRun(c3, 2, 0, 1e-5, False)
    assert np.array_equal(c2, c3)
    # npatch equal to the number of top cells, and the alternate form with many patches.
    nt = f.getNTopLevel()
    c = np.zeros((nt, 2))
    f.KMeansInitTree(c, nt, 11)
    close_centres(c, of.kmeans_init(nt, "tree", 11))
    # Errors: wrong sizes, too many patches.
    with pytest.raises(ValueError):
        f.KMeansAssign(c, nt, np.zeros(499, dtype=np.int64))
    with pytest.raises(NotImplementedError):
        big = np.zeros((6000, 2))
        f.KMeansInitTree(big, 6000, 1)
    # Empty inputs of QuickAssign.
    q = np.zeros(0, dtype=np.int64)
    T.QuickAssign(c2, 2, np.zeros(0), np.zeros(0), np.array([]), q)
