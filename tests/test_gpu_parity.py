"""GPU parity: the CUDA path (through the C ABI via the _treecorr mirror) against the
reference's golden outputs and the oracle."""
import numpy as np
import pytest

import helpers as H
from cases import CASES, flat_catalog, sphere_catalog

pytestmark = pytest.mark.gpu

# xi tolerance of the plain GPU path at equal bin_slop, relative to the array's scale.
RTOL = 1e-5


def _run_case(T, name):
    s, c1, c2, bins, min_size, max_size, ref = H.load_case(name)
    f1, f2 = H.case_fields(lambda *a: H.gpu_field(T, *a), s, c1, c2, min_size, max_size)
    got = H.gpu_process(T, s["dtype"], s["metric"], bins, f1, f2)
    return s, got, ref, f1


@pytest.mark.parametrize("name", sorted(CASES))
def test_golden(gpu_lib, name):
    s, got, ref, f1 = _run_case(gpu_lib, name)
    H.assert_outputs_close(got, ref, s["dtype"], rtol=RTOL, label=name)


@pytest.mark.parametrize("name", ["gg_flat_bs1", "gg_sphere_arc", "nn_3d", "gg_flat_middle",
                                  "gg_flat_median", "gg_flat_clumped", "vv_sphere", "tt_sphere",
                                  "qq_3d", "zz_sphere"])
def test_tree_matches_oracle(gpu_lib, name):
    """Same cells (membership, centre, size, weight, payload) as the reference rules."""
    s, c1, c2, bins, min_size, max_size, ref = H.load_case(name)
    f = H.gpu_field(gpu_lib, s["dtype"], s["coords"], c1, min_size, max_size, s["split"],
                    s["brute"], s["min_top"], s["max_top"])
    o = H.oracle_field(s["dtype"], s["coords"], c1, min_size, max_size, s["split"], s["brute"],
                       s["min_top"], s["max_top"])
    assert f.getNTopLevel() == o.ntop()
    a, b = f._dump(), o.dump()
    assert len(a["n"]) == len(b["n"])
    np.testing.assert_array_equal(a["n"], b["n"])
    np.testing.assert_array_equal(a["start"], b["start"])
    np.testing.assert_array_equal(a["depth"], b["depth"])
    for k in ("x", "y", "z"):
        np.testing.assert_allclose(a[k], b[k], rtol=0, atol=1e-12 * max(1.0, np.abs(b[k]).max()))
    np.testing.assert_allclose(a["size"], b["size"], rtol=1e-6)
    np.testing.assert_allclose(a["w"], b["w"], rtol=1e-6)
    np.testing.assert_allclose(a["d1"], b["d1"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(a["d2"], b["d2"], rtol=1e-5, atol=1e-6)


def test_repeat_is_deterministic(gpu_lib):
    """Repeated runs give identical outputs, every array bit for bit (the reference asserts
    this at num_threads=1, tests/test_gg.py:573-574): the fixed-order expansion, on by
    default, makes every warp take the same items in every run."""
    assert gpu_lib.GetDeterministic()
    s, got1, ref, _ = _run_case(gpu_lib, "gg_flat_bs1")
    _, got2, _, _ = _run_case(gpu_lib, "gg_flat_bs1")
    for k in H.OUT_KEYS:
        assert np.array_equal(got1[k], got2[k]), k


def test_shuffle_invariance(gpu_lib):
    """Input order does not change the result (reference tests/test_gg.py:1136-1162)."""
    T = gpu_lib
    rng = np.random.default_rng(11)
    cat = flat_catalog(rng, 5000)
    perm = rng.permutation(5000)
    cat2 = {k: (v[perm] if v is not None else None) for k, v in cat.items()}
    bins = dict(min_sep=1., max_sep=30., nbins=12, bin_size=np.log(30.) / 12, b=0.0, a=0.0)
    a = H.gpu_process(T, "G", "Euclidean", bins, H.gpu_field(T, "G", "flat", cat, 0., 0.))
    b = H.gpu_process(T, "G", "Euclidean", bins, H.gpu_field(T, "G", "flat", cat2, 0., 0.))
    assert np.array_equal(a["npairs"], b["npairs"])
    for k in ("weight", "xi0", "xi1", "xi2", "xi3"):
        np.testing.assert_allclose(a[k], b[k], rtol=1e-6, atol=1e-6 * a["weight"].max())


@pytest.mark.parametrize("bs", [1.0, 0.0])
def test_larger_flat_vs_oracle(gpu_lib, bs):
    """50k flat points, deep trees, many top cells: GPU vs oracle."""
    T = gpu_lib
    rng = np.random.default_rng(77)
    cat = flat_catalog(rng, 50000, L=1000.)
    nb, lo, hi = 20, 1., 100.
    bsz = np.log(hi / lo) / nb
    bins = dict(min_sep=lo, max_sep=hi, nbins=nb, bin_size=bsz, b=bs * bsz, a=0.1)
    b1 = min(0.1, bins["b"])
    mn, mx = lo * b1 / (2 + 3 * b1), hi * b1
    got = H.gpu_process(T, "G", "Euclidean", bins, H.gpu_field(T, "G", "flat", cat, mn, mx))
    ref = H.oracle_process("G", "Euclidean", bins, H.oracle_field("G", "flat", cat, mn, mx))
    H.assert_outputs_close(got, ref, "G", rtol=RTOL, label=f"flat50k bs={bs}")


def test_larger_sphere_arc_vs_oracle(gpu_lib):
    T = gpu_lib
    rng = np.random.default_rng(78)
    cat = sphere_catalog(rng, 30000, radius_deg=3.0)
    nb = 15
    lo, hi = np.radians(1. / 60), np.radians(60. / 60)
    bsz = np.log(hi / lo) / nb
    bins = dict(min_sep=lo, max_sep=hi, nbins=nb, bin_size=bsz, b=0.1 * bsz, a=0.1)
    got = H.gpu_process(T, "G", "Arc", bins, H.gpu_field(T, "G", "spherical", cat, 0., 0.))
    ref = H.oracle_process("G", "Arc", bins, H.oracle_field("G", "spherical", cat, 0., 0.))
    H.assert_outputs_close(got, ref, "G", rtol=RTOL, label="sphere30k")


@pytest.mark.parametrize("pair,geom", [("NG", "spherical"), ("KV", "flat"), ("TT", "3d"),
                                       ("QQ", "spherical"), ("NK", "spherical"),
                                       ("KZ", "3d")])
def test_other_classes_vs_oracle(gpu_lib, pair, geom):
    """The mixed and spin-s classes on 20-30K-point catalogs (cross for mixed kinds, auto for
    XX): GPU vs oracle."""
    from cases import threed_catalog
    T = gpu_lib
    rng = np.random.default_rng(sum(map(ord, pair + geom)))
    if geom == "spherical":
        mk = lambda n: sphere_catalog(rng, n, radius_deg=3.0)   # noqa: E731
        lo, hi, metric = np.radians(1. / 60), np.radians(60. / 60), "Arc"
    elif geom == "flat":
        mk = lambda n: flat_catalog(rng, n, L=600.)   # noqa: E731
        lo, hi, metric = 1., 60., "Euclidean"
    else:
        mk = lambda n: threed_catalog(rng, n, L=300.)   # noqa: E731
        lo, hi, metric = 1., 60., "Euclidean"
    nb = 12
    bsz = np.log(hi / lo) / nb
    bins = dict(min_sep=lo, max_sep=hi, nbins=nb, bin_size=bsz, b=0.2 * bsz, a=0.1)
    mn, mx = (0., 0.) if metric == "Arc" else (lo * 0.02 / 2.06, hi * 0.02)
    d1, d2 = pair[0], pair[1]
    c1 = mk(20000)
    c2 = mk(25000) if d1 != d2 else None
    g1 = H.gpu_field(T, d1, geom, c1, mn, mx)
    o1 = H.oracle_field(d1, geom, c1, mn, mx)
    g2 = H.gpu_field(T, d2, geom, c2, mn, mx) if c2 is not None else None
    o2 = H.oracle_field(d2, geom, c2, mn, mx) if c2 is not None else None
    dt = pair if d1 != d2 else d1
    got = H.gpu_process(T, dt, metric, bins, g1, g2)
    ref = H.oracle_process(dt, metric, bins, o1, o2)
    H.assert_outputs_close(got, ref, dt, rtol=RTOL, label=f"{pair} {geom}")


def test_quick_mode(gpu_lib):
    """corr_only: only weight and xi are accumulated (src/Corr2.cpp:531-551)."""
    T = gpu_lib
    s, c1, c2, bins, min_size, max_size, ref = H.load_case("gg_flat_bs1")
    f = H.gpu_field(T, "G", "flat", c1, min_size, max_size)
    got = H.gpu_process(T, "G", "Euclidean", bins, f, quick=True)
    assert not got["npairs"].any() and not got["meanr"].any() and not got["meanlogr"].any()
    np.testing.assert_allclose(got["weight"], ref["weight"], rtol=RTOL)
    np.testing.assert_allclose(got["xi0"], ref["xi0"], rtol=1e-4, atol=RTOL * np.abs(ref["xi0"]).max())


def test_accumulates_into_outputs(gpu_lib):
    """Process calls add into the caller's arrays (the reference never clears them)."""
    T = gpu_lib
    import sys
    s, c1, c2, bins, min_size, max_size, ref = H.load_case("nn_flat_bs1")
    f = H.gpu_field(T, "N", "flat", c1, min_size, max_size)
    nb = bins["nbins"]
    out = {k: np.zeros(nb) for k in H.OUT_KEYS}
    e = np.array([])
    corr = T.NNCorr(T.Log, bins["min_sep"], bins["max_sep"], nb, bins["bin_size"], bins["b"],
                    bins["a"], -sys.float_info.max, sys.float_info.max, 0., 0., 0., e, e, e, e,
                    out["meanr"], out["meanlogr"], out["weight"], out["npairs"])
    corr.processAuto(f, False, False, T.Euclidean)
    corr.processAuto(f, False, False, T.Euclidean)
    assert np.array_equal(out["npairs"], 2 * ref["npairs"])


def test_edge_cases(gpu_lib):
    T = gpu_lib
    bins = dict(min_sep=1., max_sep=10., nbins=5, bin_size=np.log(10.) / 5, b=0.1, a=0.1)
    e = np.array([])
    # Empty field: nothing accumulated, no error.
    f0 = T.NFieldFlat(e, e, e, e, e, 0., 0., T.Mean, 0, False, 3, 10)
    assert f0.getNObj() == 0
    out = H.gpu_process(T, "N", "Euclidean", bins, f0)
    assert not out["npairs"].any()
    # One point: one top cell, no pairs.
    one = np.array([1.0])
    f1 = T.NFieldFlat(one, one, e, one, e, 0., 0., T.Mean, 0, False, 3, 10)
    assert f1.getNTopLevel() == 1
    assert not H.gpu_process(T, "N", "Euclidean", bins, f1)["npairs"].any()
    # Duplicated positions (4 copies of each point), all weights positive: list leaves and
    # split duplicates count the same pairs, so npairs is exact.
    rng = np.random.default_rng(3)
    x = np.repeat(rng.uniform(0, 20, 50), 4)
    y = np.repeat(rng.uniform(0, 20, 50), 4)
    w = rng.uniform(0.5, 1.5, 200)
    cat = dict(x=x, y=y, z=None, w=w)
    for bs in (0.0, 1.0):
        b = dict(bins, b=bs * bins["bin_size"])
        got = H.gpu_process(T, "N", "Euclidean", b, H.gpu_field(T, "N", "flat", cat, 0., 0.))
        ref = H.oracle_process("N", "Euclidean", b, H.oracle_field("N", "flat", cat, 0., 0.))
        H.assert_outputs_close(got, ref, "N", label=f"dups bs={bs}")
    # Zero weights on distinct points: such points are skipped (src/Corr2.cpp:315).
    xz = rng.uniform(0, 20, 300)
    yz = rng.uniform(0, 20, 300)
    wz = rng.uniform(0.5, 1.5, 300)
    wz[::7] = 0.
    catz = dict(x=xz, y=yz, z=None, w=wz)
    for bs in (0.0, 1.0):
        b = dict(bins, b=bs * bins["bin_size"])
        got = H.gpu_process(T, "N", "Euclidean", b, H.gpu_field(T, "N", "flat", catz, 0., 0.))
        ref = H.oracle_process("N", "Euclidean", b, H.oracle_field("N", "flat", catz, 0., 0.))
        H.assert_outputs_close(got, ref, "N", label=f"zero-w bs={bs}")
    # Duplicates together with zero weights: whether exact duplicates end as one list leaf
    # or as single points depends on the last bit of their centroid, so only the weighted
    # sums (which do not depend on the tree) are compared.
    w2 = w.copy()
    w2[::7] = 0.
    cat2 = dict(x=x, y=y, z=None, w=w2)
    got = H.gpu_process(T, "N", "Euclidean", bins, H.gpu_field(T, "N", "flat", cat2, 0., 0.))
    ref = H.oracle_process("N", "Euclidean", bins, H.oracle_field("N", "flat", cat2, 0., 0.))
    H.assert_outputs_close(got, ref, "N", exact_npairs=False, label="dups+zero-w")
    # Cross with fields far apart: the early exit leaves the outputs untouched.
    far = dict(x=x + 1e4, y=y, z=None, w=w)
    got = H.gpu_process(T, "N", "Euclidean", bins, H.gpu_field(T, "N", "flat", cat, 0., 0.),
                        H.gpu_field(T, "N", "flat", far, 0., 0.))
    assert not got["weight"].any()


def test_unsupported_raise(gpu_lib):
    T = gpu_lib
    import sys
    e = np.array([])
    z = np.zeros(3)
    with pytest.raises(NotImplementedError):
        T.NNCorr(T.Linear, 1., 10., 5, 1.8, 0., 0., -sys.float_info.max, sys.float_info.max,
                 0., 0., 0., e, e, e, e, np.zeros(5), np.zeros(5), np.zeros(5), np.zeros(5))
    with pytest.raises(NotImplementedError):
        T.NFieldFlat(z, z, e, z + 1, e, 0., 0., T.Random, 0, False, 3, 10)


def test_mixed_class_arguments(gpu_lib):
    """The class fixes the two data kinds: an auto correlation of a mixed class, or fields of
    other kinds, are refused (the reference's Python never builds them)."""
    T = gpu_lib
    s, c1, c2, bins, min_size, max_size, ref = H.load_case("ng_flat_cross")
    fn = H.gpu_field(T, "N", "flat", c1, min_size, max_size)
    fg = H.gpu_field(T, "G", "flat", c2, min_size, max_size)
    fk = H.gpu_field(T, "K", "flat", c2, min_size, max_size)
    with pytest.raises(ValueError):
        H.gpu_process(T, "NG", "Euclidean", bins, fn)            # auto of a mixed class
    with pytest.raises(ValueError):
        H.gpu_process(T, "NG", "Euclidean", bins, fn, fk)        # K field as the G side
    with pytest.raises(ValueError):
        H.gpu_process(T, "NG", "Euclidean", bins, fg, fn)        # kinds swapped
    got = H.gpu_process(T, "NG", "Euclidean", bins, fn, fg)
    H.assert_outputs_close(got, ref, "NG", rtol=RTOL, label="ng after refusals")


def test_pinned_host_columns_equal_pageable(gpu_lib):
    """Page-locked host columns are read by the GPU in place, pageable ones through a staging
    copy: the same field and the same correlation, bit for bit."""
    import torch
    T = gpu_lib
    s, c1, c2, bins, min_size, max_size, ref = H.load_case("gg_sphere_arc")
    pinned = {k: (torch.from_numpy(np.ascontiguousarray(v)).pin_memory().numpy()
                  if v is not None else None) for k, v in c1.items()}
    fa = H.gpu_field(T, "G", "spherical", c1, min_size, max_size)
    fb = H.gpu_field(T, "G", "spherical", pinned, min_size, max_size)
    a = H.gpu_process(T, "G", "Arc", bins, fa)
    b = H.gpu_process(T, "G", "Arc", bins, fb)
    for k in H.OUT_KEYS:
        assert np.array_equal(a[k], b[k]), k
    H.assert_outputs_close(b, ref, "G", rtol=RTOL, label="pinned columns")
