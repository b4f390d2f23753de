"""GPU tests of the leaf-pair tiles (the exact mode: angle_slop 0, or brute fields).

In that mode the reference accepts only pairs of leaves (src/Corr2.cpp:308-389 with
include/BinType.h:93-151: s1 + s2 <= a r needs s1 + s2 = 0 when a = 0), so the GPU stops the
tree walk at cell pairs of at most 48 points per side and evaluates every leaf pair of such a
tile in k_tiles.  The tests compare the tile path with the reference's outputs, with the
traversal walked down to the leaves (TCGPU_TILES=0), and with the oracle on edge cases (list
leaves of coincident points, zero weights, self tiles, cross fields).
"""
import numpy as np
import pytest

import helpers as H
from cases import CASES, flat_catalog, sphere_catalog, threed_catalog

pytestmark = pytest.mark.gpu
RTOL = 1e-5

EXACT = sorted(n for n, c in CASES.items() if c[10] == 0.0 or c[12])


@pytest.mark.parametrize("name", EXACT)
@pytest.mark.parametrize("tiles", ["1", "0"])
def test_exact_golden_both_paths(gpu_lib, monkeypatch, name, tiles):
    monkeypatch.setenv("TCGPU_TILES", tiles)
    T = gpu_lib
    s, c1, c2, bins, min_size, max_size, ref = H.load_case(name)
    f1, f2 = H.case_fields(lambda *a: H.gpu_field(T, *a), s, c1, c2, min_size, max_size)
    got = H.gpu_process(T, s["dtype"], s["metric"], bins, f1, f2)
    H.assert_outputs_close(got, ref, s["dtype"], rtol=RTOL, label=f"{name} tiles={tiles}")
    st = got["_stats"]
    if tiles == "1":
        assert st["tiles"] > 0
    else:
        assert st["tiles"] == 0


def _exact_vs_oracle(T, dtype, coords, metric, bins, c1, c2=None, label=""):
    g1 = H.gpu_field(T, dtype[0], coords, c1, 0., 0.)
    o1 = H.oracle_field(dtype[0], coords, c1, 0., 0.)
    g2 = H.gpu_field(T, dtype[-1], coords, c2, 0., 0.) if c2 is not None else None
    o2 = H.oracle_field(dtype[-1], coords, c2, 0., 0.) if c2 is not None else None
    got = H.gpu_process(T, dtype, metric, bins, g1, g2)
    ref = H.oracle_process(dtype, metric, bins, o1, o2)
    H.assert_outputs_close(got, ref, dtype, rtol=RTOL, label=label)
    return got


@pytest.mark.parametrize("dtype,coords", [("G", "flat"), ("G", "spherical"), ("N", "3d"),
                                          ("K", "spherical"), ("V", "flat"), ("Q", "3d")])
def test_exact_larger_vs_oracle(gpu_lib, dtype, coords):
    """20-40K points in exact mode, deep trees, many tiles: GPU tiles vs the oracle."""
    T = gpu_lib
    rng = np.random.default_rng(sum(map(ord, dtype + coords)) + 17)
    if coords == "flat":
        cat, metric, lo, hi = flat_catalog(rng, 40000, L=400.), "Euclidean", 1., 60.
    elif coords == "spherical":
        cat, metric = sphere_catalog(rng, 30000, radius_deg=3.0), "Arc"
        lo, hi = np.radians(1. / 60), np.radians(90. / 60)
    else:
        cat, metric, lo, hi = threed_catalog(rng, 20000, L=200.), "Euclidean", 1., 40.
    nb = 16
    bsz = np.log(hi / lo) / nb
    bins = dict(min_sep=lo, max_sep=hi, nbins=nb, bin_size=bsz, b=0.0, a=0.0)
    got = _exact_vs_oracle(T, dtype, coords, metric, bins, cat, label=f"exact {dtype} {coords}")
    assert got["_stats"]["tiles"] > 0


def test_exact_cross_mixed_vs_oracle(gpu_lib):
    T = gpu_lib
    rng = np.random.default_rng(91)
    c1, c2 = sphere_catalog(rng, 15000, radius_deg=2.0), sphere_catalog(rng, 18000, radius_deg=2.0)
    lo, hi = np.radians(0.5 / 60), np.radians(60. / 60)
    nb = 12
    bins = dict(min_sep=lo, max_sep=hi, nbins=nb, bin_size=np.log(hi / lo) / nb, b=0.0, a=0.0)
    for dt in ("NG", "KG", "NK"):
        _exact_vs_oracle(T, dt, "spherical", "Arc", bins, c1, c2, label=f"exact cross {dt}")


def test_exact_edge_cases(gpu_lib):
    """List leaves of coincident points (a leaf with n > 1 inside a tile), zero weights, and a
    catalog smaller than one tile."""
    T = gpu_lib
    rng = np.random.default_rng(4)
    bins = dict(min_sep=0.5, max_sep=15., nbins=8, bin_size=np.log(30.) / 8, b=0.0, a=0.0)
    x = np.repeat(rng.uniform(0, 20, 400), 3)
    y = np.repeat(rng.uniform(0, 20, 400), 3)
    n = len(x)
    cat = dict(x=x, y=y, z=None, g1=rng.normal(0, .2, n), g2=rng.normal(0, .2, n),
               k=rng.normal(0, .02, n), w=rng.uniform(0.5, 1.5, n))
    _exact_vs_oracle(T, "G", "flat", "Euclidean", bins, cat, label="exact duplicates")
    catz = dict(cat, x=rng.uniform(0, 20, n), y=rng.uniform(0, 20, n))
    catz["w"] = catz["w"].copy()
    catz["w"][::5] = 0.
    _exact_vs_oracle(T, "K", "flat", "Euclidean", bins, catz, label="exact zero weights")
    small = {k: (v[:20] if v is not None else None) for k, v in catz.items()}
    _exact_vs_oracle(T, "N", "flat", "Euclidean", bins, small, label="exact 20 points")


def test_exact_tiles_agree_with_traversal(gpu_lib, monkeypatch):
    """The same exact-mode correlation with tiles and with the traversal walked down to the
    leaves: identical pair counts and sums within FP32 rounding."""
    T = gpu_lib
    rng = np.random.default_rng(23)
    cat = sphere_catalog(rng, 60000, radius_deg=4.0)
    lo, hi = np.radians(1. / 60), np.radians(120. / 60)
    nb = 20
    bins = dict(min_sep=lo, max_sep=hi, nbins=nb, bin_size=np.log(hi / lo) / nb, b=0.0, a=0.0)
    f = H.gpu_field(T, "G", "spherical", cat, 0., 0.)
    monkeypatch.setenv("TCGPU_TILES", "1")
    a = H.gpu_process(T, "G", "Arc", bins, f)
    monkeypatch.setenv("TCGPU_TILES", "0")
    b = H.gpu_process(T, "G", "Arc", bins, f)
    assert a["_stats"]["tiles"] > 0 and b["_stats"]["tiles"] == 0
    H.assert_outputs_close(a, b, "G", rtol=2e-6, label="tiles vs traversal")


@pytest.mark.parametrize("dtype,coords,metric", [("G", "spherical", "Euclidean"),
                                                 ("G", "3d", "Euclidean"),
                                                 ("T", "spherical", "Arc")])
def test_exact_other_geometries_vs_oracle(gpu_lib, dtype, coords, metric):
    """The tile kernel's other geometry instantiations: sphere with the Euclidean (chord)
    metric, 3-d GG (the generic projection), spin-3 on the sphere."""
    T = gpu_lib
    rng = np.random.default_rng(sum(map(ord, dtype + coords + metric)))
    if coords == "spherical":
        cat = sphere_catalog(rng, 25000, radius_deg=3.0)
        lo, hi = np.radians(1. / 60), np.radians(90. / 60)
    else:
        cat, lo, hi = threed_catalog(rng, 20000, L=200.), 1., 40.
    nb = 14
    bins = dict(min_sep=lo, max_sep=hi, nbins=nb, bin_size=np.log(hi / lo) / nb, b=0.0, a=0.0)
    got = _exact_vs_oracle(T, dtype, coords, metric, bins, cat,
                           label=f"exact {dtype} {coords} {metric}")
    assert got["_stats"]["tiles"] > 0


def test_exact_negative_weights_and_quick(gpu_lib):
    """Negative weights (cells whose sums stay non-zero) and corr_only (quick: no npairs,
    meanr or meanlogr) through the tiles."""
    T = gpu_lib
    rng = np.random.default_rng(31)
    cat = flat_catalog(rng, 30000, L=300.)
    cat["w"] = cat["w"] * np.where(rng.uniform(size=len(cat["w"])) < 0.3, -1., 1.)
    lo, hi, nb = 1., 50., 12
    bins = dict(min_sep=lo, max_sep=hi, nbins=nb, bin_size=np.log(hi / lo) / nb, b=0.0, a=0.0)
    _exact_vs_oracle(T, "G", "flat", "Euclidean", bins, cat, label="exact negative weights")
    g = H.gpu_field(T, "G", "flat", cat, 0., 0.)
    o = H.oracle_field("G", "flat", cat, 0., 0.)
    got = H.gpu_process(T, "G", "Euclidean", bins, g, quick=True)
    ref = H.oracle_process("G", "Euclidean", bins, o, quick=True)
    assert not got["npairs"].any() and not got["meanr"].any()
    for k in ("weight", "xi0", "xi1", "xi2", "xi3"):
        scale = max(np.abs(ref[k]).max(), 1e-300)
        assert np.abs(got[k] - ref[k]).max() <= RTOL * scale, k
