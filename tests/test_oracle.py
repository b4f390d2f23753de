"""CPU tests: the oracle against the reference's golden outputs (the parity pin)."""
import numpy as np
import pytest

import helpers as H
from cases import CASES


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference(name):
    s, c1, c2, bins, min_size, max_size, ref = H.load_case(name)
    f1, f2 = H.case_fields(H.oracle_field, s, c1, c2, min_size, max_size)
    out = H.oracle_process(s["dtype"], s["metric"], bins, f1, f2, nthreads=1)
    assert np.array_equal(out["npairs"], ref["npairs"])
    for k in H.OUT_KEYS:
        r = ref[k]
        scale = max(np.abs(r).max(), 1e-300)
        assert np.abs(out[k] - r).max() <= 1e-12 * scale, k


def test_oracle_brute_force_flat():
    """Independent FP64 brute force (the math of tests/test_gg.py:58-77 of the reference):
    with bin_slop=0 and angle_slop=0 the tree result equals the all-pairs sum."""
    from cases import flat_catalog
    rng = np.random.default_rng(5)
    cat = flat_catalog(rng, 600)
    nb, lo, hi = 8, 2.0, 30.0
    bins = dict(min_sep=lo, max_sep=hi, nbins=nb, bin_size=np.log(hi / lo) / nb, b=0.0, a=0.0)
    f = H.oracle_field("G", "flat", cat, 0.0, 0.0)
    out = H.oracle_process("G", "Euclidean", bins, f, nthreads=1)
    x, y, w = cat["x"], cat["y"], cat["w"]
    g = (cat["g1"] + 1j * cat["g2"]) * w
    i, j = np.triu_indices(len(x), 1)
    dx, dy = x[j] - x[i], y[j] - y[i]
    r = np.hypot(dx, dy)
    ok = (r >= lo) & (r < hi)
    i, j, dx, dy, r = i[ok], j[ok], dx[ok], dy[ok], r[ok]
    k = np.floor(np.log(r / lo) / bins["bin_size"]).astype(int)
    e = ((dx - 1j * dy) / r) ** 2      # exp(-2i alpha), alpha = angle of p2 - p1
    g1, g2 = g[i] * e, g[j] * e
    np_ = np.bincount(k, minlength=nb)
    xip = np.bincount(k, (g1 * np.conj(g2)).real, minlength=nb)
    xim = np.bincount(k, (g1 * g2).real, minlength=nb)
    ww = np.bincount(k, w[i] * w[j], minlength=nb)
    assert np.array_equal(out["npairs"], np_.astype(float))
    np.testing.assert_allclose(out["weight"], ww, rtol=1e-6)
    np.testing.assert_allclose(out["xi0"], xip, rtol=1e-5, atol=1e-6 * ww.max())
    np.testing.assert_allclose(out["xi2"], xim, rtol=1e-5, atol=1e-6 * ww.max())


@pytest.mark.parametrize("name", ["ggg_flat_mp", "ggg_flat_mp_n20", "ggg_flat_mp_bs0",
                                  "ggg_sphere_mp"])
def test_oracle_multipole_matches_reference(name):
    """GGG LogMultipole: the oracle's restatement against the reference's own outputs."""
    import os
    from cases3 import spec3
    from oracle import oracle as O
    s = spec3(name)
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    c = {k[3:]: g[k] for k in g.files if k.startswith("c1_")}
    f = O.OracleField("G", s["coords"], c["x"], c["y"], c.get("z"), c["g1"], c["g2"], c["w"],
                      None, float(g["min_size"]), float(g["max_size"]), "mean", False, 3, 10)
    bins = dict(min_sep=s["min_sep"], max_sep=s["max_sep"], nbins=s["nbins"],
                bin_size=s["bin_size"], b=s["b"], a=s["a"])
    out = O.multipole(s["metric"], bins, s["max_n"], f, nthreads=1)
    assert np.array_equal(out["ntri"], g["ref_ntri"])
    for k in O.MP_KEYS:
        r = g["ref_" + k]
        assert np.abs(out[k] - r).max() <= 1e-12 * max(np.abs(r).max(), 1e-300), k


@pytest.mark.parametrize("name", ["nnn_flat_mp", "nnn_sphere_mp"])
def test_oracle_multipole_nnn_matches_reference(name):
    """NNN LogMultipole (the reference's NNNCorr): its weight, ntri and mean distances are
    the multipole sums that do not depend on the payload, so the oracle's multipole on the
    same points with zero shears reproduces them."""
    import os
    from cases3 import spec3
    from oracle import oracle as O
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    s = spec3(str(g["case"]))
    c = {k[3:]: g[k] for k in g.files if k.startswith("c1_")}
    zero = np.zeros(len(c["x"]))
    f = O.OracleField("G", s["coords"], c["x"], c["y"], c.get("z"), zero, zero, c["w"],
                      None, float(g["min_size"]), float(g["max_size"]), "mean", False, 3, 10)
    bins = dict(min_sep=s["min_sep"], max_sep=s["max_sep"], nbins=s["nbins"],
                bin_size=s["bin_size"], b=s["b"], a=s["a"])
    out = O.multipole(s["metric"], bins, s["max_n"], f, nthreads=1)
    assert np.array_equal(out["ntri"], g["ref_ntri"])
    for k in ("weight", "weight_im", "meand2", "meanlogd2", "meand3", "meanlogd3"):
        r = g["ref_" + k]
        assert np.abs(out[k] - r).max() <= 1e-12 * max(np.abs(r).max(), 1e-300), k


@pytest.mark.parametrize("name", ["kkk_flat_mp", "kkk_sphere_mp"])
def test_oracle_multipole_kkk_identity(name):
    """KKK LogMultipole (the reference's KKKCorr): its zeta is the multipole weight
    contraction with every weight w replaced by w k (src/Corr3.cpp:1912-1965 against
    MultipoleHelper<1>, 2108-2150), so the oracle's multipole with weights w k, position
    weights w and no shear reproduces it; weight and ntri come from the plain weights."""
    import os
    from cases3 import spec3
    from oracle import oracle as O
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    s = spec3(str(g["case"]))
    c = {k[3:]: g[k] for k in g.files if k.startswith("c1_")}
    zero = np.zeros(len(c["x"]))
    bins = dict(min_sep=s["min_sep"], max_sep=s["max_sep"], nbins=s["nbins"],
                bin_size=s["bin_size"], b=s["b"], a=s["a"])
    args = (float(g["min_size"]), float(g["max_size"]), "mean", False, 3, 10)
    fk = O.OracleField("G", s["coords"], c["x"], c["y"], c.get("z"), zero, zero,
                       c["w"] * c["k"], c["w"], *args)
    zk = O.multipole(s["metric"], bins, s["max_n"], fk, nthreads=1)
    for mine, ref in (("weight", "zeta"), ("weight_im", "zeta_im")):
        r = g["ref_" + ref]
        assert np.abs(zk[mine] - r).max() <= 1e-12 * max(np.abs(r).max(), 1e-300), ref
    fw = O.OracleField("G", s["coords"], c["x"], c["y"], c.get("z"), zero, zero, c["w"], None,
                       *args)
    ww = O.multipole(s["metric"], bins, s["max_n"], fw, nthreads=1)
    assert np.array_equal(ww["ntri"], g["ref_ntri"])
    for k in ("weight", "weight_im", "meand2", "meanlogd2", "meand3", "meanlogd3"):
        r = g["ref_" + k]
        assert np.abs(ww[k] - r).max() <= 1e-12 * max(np.abs(r).max(), 1e-300), k


X12 = ["ggg_flat_mp_x12", "ggg_sphere_mp_x12", "nnn_flat_mp_x12", "kkk_sphere_mp_x12",
       "nkk_flat_mp_x12", "knn_sphere_mp_x12", "ngg_flat_mp_x12", "ngg_sphere_mp_x12",
       "kgg_sphere_mp_x12", "gnn_flat_mp_x12", "gnn_sphere_mp_x12", "gkk_sphere_mp_x12"]


@pytest.mark.parametrize("name", X12)
def test_oracle_multipole_cross12_matches_reference(name):
    """processCross12 (ordered = 1) with LogMultipole: vertex 1 from the first catalog,
    vertices 2 and 3 from the second (src/Corr3.cpp:1177-1237).  The N and K classes go
    through the identities of their auto-correlations: weight, ntri and the mean distances
    do not depend on the payload, and zeta (MultipoleHelper<1>, 2108-2214) is the weight
    contraction with every K point's weight w replaced by w k."""
    import os
    from cases3 import spec3
    from oracle import oracle as O
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    s = spec3(str(g["case"]))
    letters = str(g["letters"])
    bins = dict(min_sep=s["min_sep"], max_sep=s["max_sep"], nbins=s["nbins"],
                bin_size=s["bin_size"], b=s["b"], a=s["a"])
    args = (float(g["min_size"]), float(g["max_size"]), "mean", False, 3, 10)
    cats = [{k[3:]: g[k] for k in g.files if k.startswith(p)} for p in ("c1_", "c2_")]

    def field(c, kind, wk):
        zero = np.zeros(len(c["x"]))
        if kind == "G":
            return O.OracleField("G", s["coords"], c["x"], c["y"], c.get("z"), c["g1"], c["g2"],
                                 c["w"], None, *args)
        w, wpos = (c["w"] * c["k"], c["w"]) if (wk and kind == "K") else (c["w"], None)
        return O.OracleField("G", s["coords"], c["x"], c["y"], c.get("z"), zero, zero, w, wpos,
                             *args)

    def close(a, r, what):
        assert np.abs(a - r).max() <= 1e-12 * max(np.abs(r).max(), 1e-300), what

    real = "K" in letters and "G" not in letters     # KKK, NKK, KNN
    vreal = (letters[0] != "G" and letters[1] == "G") or real
    pspin0 = (letters[0] == "G" and letters[1] != "G") or real

    def as_k(c, letter):
        # An N or K catalog as a K field whose k is 1 (N) or k (K): its cells' d1 is the
        # real payload w or w k, summed without parallel transport.
        kv = c["k"] if letter == "K" else np.ones(len(c["x"]))
        return O.OracleField("K", s["coords"], c["x"], c["y"], c.get("z"), kv, None, c["w"],
                             None, *args)

    f1 = as_k(cats[0], letters[0]) if vreal else field(cats[0], letters[0], False)
    f2 = as_k(cats[1], letters[1]) if pspin0 else field(cats[1], letters[1], False)
    mode = 3 if real else 1 if vreal else 2 if pspin0 else 0
    out = O.multipole(s["metric"], bins, s["max_n"], f1, nthreads=1, f2=f2, mode=mode)
    assert np.array_equal(out["ntri"], g["ref_ntri"])
    assert out["ntri"].sum() > 0
    for k in ("weight", "weight_im", "meand2", "meanlogd2", "meand3", "meanlogd3"):
        close(out[k], g["ref_" + k], k)
    if letters == "GGG":
        for k in O.MP_KEYS[:8]:
            close(out[k], g["ref_" + k], k)
    if vreal and not real:
        # MultipoleHelper<2>'s zeta0 and zeta1 are the contraction's gam0 and gam2.
        for mine, ref in (("gam0r", "gam0r"), ("gam0i", "gam0i"), ("gam2r", "gam1r"),
                          ("gam2i", "gam1i")):
            close(out[mine], g["ref_" + ref], ref)
    elif pspin0:
        # MultipoleHelper<4>'s and <1>'s zeta is the contraction's gam0.
        close(out["gam0r"], g["ref_zeta"], "zeta")
        close(out["gam0i"], g["ref_zeta_im"], "zeta_im")
    if real:
        # The same zeta as the weight contraction over the weights w k (the identity the
        # KKK auto test checks).
        k1, k2 = field(cats[0], letters[0], True), field(cats[1], letters[1], True)
        zk = O.multipole(s["metric"], bins, s["max_n"], k1, nthreads=1, f2=k2)
        close(zk["weight"], g["ref_zeta"], "zeta")
        close(zk["weight_im"], g["ref_zeta_im"], "zeta_im")


X3 = ["ggg_flat_mp_x3o4", "ggg_sphere_mp_x3o1", "ggg_flat_mp_x21o3", "kkk_flat_mp_x3o0",
      "nnn_sphere_mp_x12o0", "ngg_flat_mp_x3o4", "gkk_sphere_mp_x3o1", "nnk_flat_mp_x21o3",
      "nkn_sphere_mp_x3o4", "knk_flat_mp_x3o4", "kkn_sphere_mp_x21o3", "nng_flat_mp_x21o3",
      "ngn_sphere_mp_x3o4", "kkg_sphere_mp_x21o3", "kgk_flat_mp_x3o4", "gng_flat_mp_x3o4",
      "ggn_sphere_mp_x21o3", "gkg_sphere_mp_x3o4", "ggk_flat_mp_x21o3", "ggg_flat_mp_x3o2",
      "nnn_flat_mp_x3o3", "kkk_sphere_mp_x21o0"]


def x3_fields(O, g, s):
    """The fixture's catalogs as oracle fields in the representation of the class (the
    identities of the cross12 test) and the oracle mode."""
    letters = str(g["letters"])
    args = (float(g["min_size"]), float(g["max_size"]), "mean", False, 3, 10)
    cats = []
    for i in (1, 2, 3):
        c = {k[3:]: g[k] for k in g.files if k.startswith(f"c{i}_")}
        if c:
            cats.append(c)

    def mk(c, rep):
        zero = np.zeros(len(c["x"]))
        if rep == "G":
            return O.OracleField("G", s["coords"], c["x"], c["y"], c.get("z"), c["g1"],
                                 c["g2"], c["w"], None, *args)
        if rep == "G0":
            return O.OracleField("G", s["coords"], c["x"], c["y"], c.get("z"), zero, zero,
                                 c["w"], None, *args)
        kv = c["k"] if rep == "K" else np.ones(len(c["x"]))
        return O.OracleField("K", s["coords"], c["x"], c["y"], c.get("z"), kv, None, c["w"],
                             None, *args)

    if letters == "GGG":
        return [mk(c, "G") for c in cats], 0
    if letters == "NNN":
        return [mk(c, "G0") for c in cats], 0
    # Every other class: each vertex's field as G (spin 2) or as a K field whose k is 1 (N)
    # or k (K); mode bit i set where vertex i+1 is real.
    kinds = {"cross": letters, "cross21": letters[0] + letters[2],
             "cross12": letters[:2]}[str(g["call"])]
    fs = [mk(c, "G" if L == "G" else "K" if L == "K" else "K1") for c, L in zip(cats, kinds)]
    mode = sum(1 << i for i, L in enumerate(letters) if L != "G")
    return fs, mode


def x3_oracle(O, g, s):
    """The reference's dispatch of processCross / processCross21 / processCross12
    (src/Corr3.cpp:3938-3976, 3831-3868, 3730-3768) over the oracle's multipoles."""
    fs, mode = x3_fields(O, g, s)
    bins = dict(min_sep=s["min_sep"], max_sep=s["max_sep"], nbins=s["nbins"],
                bin_size=s["bin_size"], b=s["b"], a=s["a"])
    call, ordered = str(g["call"]), int(g["ordered"])
    out = {k: np.zeros((s["nbins"], s["nbins"], 2 * s["max_n"] + 1)) for k in O.MP_KEYS}

    def m3(a, b, c, o):
        O.multipole3(s["metric"], bins, s["max_n"], a, b, c, o, nthreads=1, mode=mode, out=out)

    if call == "cross":
        f1, f2, f3 = fs
        if ordered == 0:
            m3(f2, f1, f3, 1); m3(f3, f1, f2, 1); m3(f1, f2, f3, 1)
        elif ordered == 1:
            m3(f1, f2, f3, 1)
        elif ordered == 2:
            m3(f1, f2, f3, 4); m3(f3, f2, f1, 4)
        elif ordered == 3:
            m3(f1, f2, f3, 4); m3(f2, f1, f3, 4)
        else:
            m3(f1, f2, f3, 4)
    elif call == "cross21":
        f1, f2 = fs
        if ordered == 0:
            m3(f2, f1, f1, 1); m3(f1, f2, f1, 1); m3(f1, f1, f2, 1)
        else:
            m3(f1, f1, f2, 4)
    else:
        f1, f2 = fs
        if ordered == 0:
            m3(f2, f1, f2, 1)
        o2 = O.multipole(s["metric"], bins, s["max_n"], f1, nthreads=1, f2=f2, mode=mode)
        for k in O.MP_KEYS:
            out[k] += o2[k]
    return out


def x3_zeta_pairs(letters):
    """(oracle output, reference output) pairs of the class's zeta arrays: GGG's gam0..3;
    N/K-vertex with two G's (MultipoleHelper<2>): gam0, gam2; G-vertex with one G
    (MultipoleHelper<6>): gam0, gam1; every class with one or no G: gam0 as zeta."""
    nG = letters.count("G")
    if nG == 3:
        return [(k, k) for k in ("gam0r", "gam0i", "gam1r", "gam1i", "gam2r", "gam2i", "gam3r",
                                 "gam3i")]
    if letters == "NNN":
        return []
    if nG == 2 and letters[0] != "G":
        return [("gam0r", "gam0r"), ("gam0i", "gam0i"), ("gam2r", "gam1r"), ("gam2i", "gam1i")]
    if nG == 2:
        return [(k, k) for k in ("gam0r", "gam0i", "gam1r", "gam1i")]
    return [("gam0r", "zeta"), ("gam0i", "zeta_im")]


@pytest.mark.parametrize("name", X3)
def test_oracle_multipole_three_field_matches_reference(name):
    """The three-field multipole (src/Corr3.cpp:1239-1305, calculateZeta 1976-2087 with the
    reference's ordered = 1 meanlogd3 term) through the reference's dispatch of
    processCross / processCross21 / processCross12(ordered = 0)."""
    import os
    from cases3 import spec3
    from oracle import oracle as O
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    s = spec3(str(g["case"]))
    out = x3_oracle(O, g, s)
    assert np.array_equal(out["ntri"], g["ref_ntri"])
    assert out["ntri"].sum() > 0

    def close(a, r, what):
        assert np.abs(a - r).max() <= 1e-12 * max(np.abs(r).max(), 1e-300), what

    for k in ("weight", "weight_im", "meand2", "meanlogd2", "meand3", "meanlogd3"):
        close(out[k], g["ref_" + k], k)
    for mine, ref in x3_zeta_pairs(str(g["letters"])):
        close(out[mine], g["ref_" + ref], ref)
