"""CPU tests: the k-means restatement of the oracle against the reference's golden outputs
(tests/golden/km_*.npz, written by make_golden.py --kmeans from the reference module)."""
import os

import numpy as np
import pytest

from cases_km import KM_CASES, KM_MAX_ITER, KM_SEED, KM_TOL, km_spec
from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    d = np.load(os.path.join(GOLD, name + ".npz"))
    return {k: d[k] for k in d.files}


def field(name, g):
    s = km_spec(name)
    return O.OracleField("N", s["coords"], g["x"], g["y"], g.get("z"), w=g["w"],
                         min_size=0.0, max_size=np.inf, split_method="mean",
                         min_top=s["min_top"], max_top=s["max_top"])


@pytest.mark.parametrize("name", sorted(KM_CASES))
def test_kmeans_init_matches_reference(name):
    g = load(name)
    f = field(name, g)
    assert f.ntop() == int(g["ntop"])
    npatch = km_spec(name)["npatch"]
    for tag, init in (("tree", "tree"), ("rand", "random"), ("kmpp", "kmeans++")):
        c = f.kmeans_init(npatch, init, KM_SEED)
        if km_spec(name)["coords"] == "spherical":
            # The reference (built with -ffast-math) normalises ~0.6% of the unit vectors
            # with a reciprocal multiply on some components: 1 ulp.
            np.testing.assert_allclose(c, g["init_" + tag], rtol=0, atol=2.3e-16, err_msg=tag)
        else:
            assert np.array_equal(c, g["init_" + tag]), tag


@pytest.mark.parametrize("name", sorted(KM_CASES))
def test_kmeans_run_matches_reference(name):
    g = load(name)
    f = field(name, g)
    for tag, iters, alt in (("it1", 1, False), ("it3", 3, False), ("run", KM_MAX_ITER, False),
                            ("alt_it1", 1, True), ("alt_it3", 3, True),
                            ("alt_run", KM_MAX_ITER, True)):
        c, _ = f.kmeans_run(g["init_tree"], iters, KM_TOL, alt)
        # Same cells, same order of sums (one thread): equal up to the reference's
        # -ffast-math reassociation of the divisions.
        np.testing.assert_allclose(c, g[tag], rtol=0, atol=1e-12 * np.abs(g[tag]).max(),
                                   err_msg=tag)
    assert np.array_equal(f.kmeans_assign(g["run"]), g["assign"])
    assert np.array_equal(f.kmeans_assign(g["alt_run"]), g["alt_assign"])


@pytest.mark.parametrize("name", sorted(KM_CASES))
def test_quick_assign_select_patch_match_reference(name):
    g = load(name)
    z = g.get("z")
    assert np.array_equal(O.quick_assign(g["run"], g["x"], g["y"], z), g["quick"])
    npatch = km_spec(name)["npatch"]
    for pp in (0, npatch - 1):
        assert np.array_equal(O.select_patch(pp, g["run"], g["x"], g["y"], z), g["select_%d" % pp])


def test_kmeans_assign_equals_nearest_centre():
    """For the plain criterion, the tree assignment is the point-wise nearest centre."""
    g = load("km_flat")
    f = field("km_flat", g)
    assert np.array_equal(f.kmeans_assign(g["run"]), O.quick_assign(g["run"], g["x"], g["y"]))
