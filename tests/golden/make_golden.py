"""Generate the golden fixtures in tests/golden/*.npz from the reference TreeCorr C++.

Run in a container that has the reference sources (it does not run on the GPU machine):

    make -f oracle/Makefile.ref -j8 REF=$TREECORR_REFERENCE   # builds oracle/_ref/_treecorr*.so
    python tests/golden/make_golden.py

For every case in tests/golden/cases.py it builds the reference's own native Field and
Corr objects (the module `_treecorr`, exactly as treecorr/field.py and
treecorr/corr2base.py drive it) and stores the inputs next to the accumulated outputs.
The reference is run with one OpenMP thread so its summation order is fixed.
"""
import glob
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
from cases import CASES, kinds, make_inputs, spec_dict, xi_count  # noqa: E402

so = glob.glob(os.path.join(ROOT, "oracle", "_ref", "_treecorr*.so"))
if not so:
    sys.exit("reference module not built: make -f oracle/Makefile.ref -j8")
sys.path.insert(0, os.path.dirname(so[0]))
import _treecorr  # noqa: E402  (the reference's own module)

SPLIT = {"mean": _treecorr.Mean, "median": _treecorr.Median, "middle": _treecorr.Middle}
METRIC = {"Euclidean": _treecorr.Euclidean, "Arc": _treecorr.Arc}
COORDS = {"flat": "Flat", "spherical": "Sphere", "3d": "ThreeD"}


def build_field(dtype, coords, cat, min_size, max_size, split, brute, min_top, max_top):
    empty = np.array([])
    z = cat["z"] if cat["z"] is not None else empty
    cls = getattr(_treecorr, dtype + "Field" + COORDS[coords])
    args = [cat["x"], cat["y"], z]
    if dtype == "K":
        args += [cat["k"]]
    elif dtype in "ZVGTQ":
        args += [cat["g1"], cat["g2"]]
    args += [cat["w"], empty, min_size, max_size, SPLIT[split], 0, brute, min_top, max_top]
    return cls(*args)


def run_case(name):
    s = spec_dict(name)
    cat1, cat2 = make_inputs(name)
    bin_size = np.log(s["max_sep"] / s["min_sep"]) / s["nbins"]
    b = bin_size * s["bin_slop"]
    a = s["angle_slop"]
    if s["metric"] == "Euclidean":
        b1 = min(a, b)
        min_size, max_size = s["min_sep"] * b1 / (2 + 3 * b1), s["max_sep"] * b1
    else:
        min_size, max_size = 0.0, 0.0
    if s["brute"]:
        min_size = 0.0
    max_size = max_size if max_size > 0 else 0.0
    nb = s["nbins"]
    out = {k: np.zeros(nb) for k in ("xi0", "xi1", "xi2", "xi3", "meanr", "meanlogr",
                                      "weight", "npairs")}
    e = np.array([])
    d1, d2 = kinds(s["dtype"])
    nxi = xi_count(s["dtype"])
    xi = [out["xi%d" % i] if i < nxi else e for i in range(4)]
    corr = getattr(_treecorr, d1 + d2 + "Corr")(
        _treecorr.Log, s["min_sep"], s["max_sep"], nb, bin_size, b, a,
        -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
        xi[0], xi[1], xi[2], xi[3], out["meanr"], out["meanlogr"], out["weight"], out["npairs"])
    f1 = build_field(d1, s["coords"], cat1, min_size, max_size, s["split"], s["brute"],
                     s["min_top"], s["max_top"])
    if cat2 is None:
        corr.processAuto(f1, False, False, METRIC[s["metric"]])
    else:
        f2 = build_field(d2, s["coords"], cat2, min_size, max_size, s["split"],
                         s["brute"], s["min_top"], s["max_top"])
        corr.processCross(f1, f2, False, False, METRIC[s["metric"]])
    save = dict(min_size=min_size, max_size=max_size, bin_size=bin_size, b=b, a=a,
                ntop=f1.getNTopLevel())
    for k, v in cat1.items():
        if v is not None:
            save["c1_" + k] = v
    if cat2 is not None:
        for k, v in cat2.items():
            if v is not None:
                save["c2_" + k] = v
    for k, v in out.items():
        save["ref_" + k] = v
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **save)
    return out


if __name__ == "__main__" and not {"--mp", "--mp-nnn", "--mp-kkk", "--mp-x12", "--mp-x3",
                                   "--xyz", "--kmeans", "--bench"} & set(sys.argv):
    _treecorr.SetOMPThreads(1)
    names = sys.argv[1:] or list(CASES)
    for name in names:
        out = run_case(name)
        print(f"{name:24s} npairs={out['npairs'].sum():.0f} weight={out['weight'].sum():.6g}")


def run_case3(name):
    """GGG LogMultipole auto-correlation through the reference's GGGCorr (driven the way
    treecorr/corr3base.py:1116-1131 and 1870-1911 drive it)."""
    from cases3 import make_inputs3, spec3
    s = spec3(name)
    cat = make_inputs3(name)
    if s["metric"] == "Euclidean":
        b1 = min(s["a"], s["b"])
        min_size, max_size = 2 * s["min_sep"] * b1 / (2. + 3 * b1), s["max_sep"] * b1
    else:
        min_size, max_size = 0.0, 0.0
    nb, mn = s["nbins"], s["max_n"]
    shape = (nb, nb, 2 * mn + 1)
    keys = ("gam0r", "gam0i", "gam1r", "gam1i", "gam2r", "gam2i", "gam3r", "gam3i",
            "meand1", "meanlogd1", "meand2", "meanlogd2", "meand3", "meanlogd3", "meanu",
            "meanv", "weight", "weight_im", "ntri")
    out = {k: np.zeros(shape) for k in keys}
    corr = _treecorr.GGGCorr(
        _treecorr.LogMultipole, s["min_sep"], s["max_sep"], nb, s["bin_size"], s["b"], s["a"],
        0., 0., mn, 0., 0., 0., 0., 0, 0., 0.,
        -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
        *[out[k] for k in keys])
    f = build_field("G", s["coords"], cat, min_size, max_size, "mean", False, 3, 10)
    corr.processAuto(f, False, False, METRIC[s["metric"]])
    save = dict(min_size=min_size, max_size=max_size)
    for k, v in cat.items():
        if v is not None:
            save["c1_" + k] = v
    for k, v in out.items():
        save["ref_" + k] = v
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **save)
    return out


if __name__ == "__main__" and "--mp" in sys.argv:
    _treecorr.SetOMPThreads(1)
    from cases3 import CASES3
    for name in CASES3:
        out = run_case3(name)
        print(f"{name:20s} ntri={out['ntri'].sum():.6g} weight={out['weight'].sum():.6g}")


# GenerateXYZ (src/KMeans.cpp:1013-1050): ra/dec (radians), with and without a distance.
if __name__ == "__main__" and "--xyz" in sys.argv:
    rng = np.random.default_rng(20240613)
    n = 4000
    ra = rng.uniform(0, 2 * np.pi, n)
    dec = np.arcsin(rng.uniform(-1, 1, n))
    r = rng.uniform(10., 3000., n)
    out = {"ra": ra, "dec": dec, "r": r}
    for tag, rr in (("", np.array([])), ("_r", r)):
        x, y, z = np.zeros(n), np.zeros(n), np.zeros(n)
        _treecorr.GenerateXYZ(x, y, z, ra, dec, rr)
        out["x" + tag], out["y" + tag], out["z" + tag] = x, y, z
    np.savez(os.path.join(HERE, "generate_xyz.npz"), **out)
    print("generate_xyz.npz")


# k-means (src/KMeans.cpp): the three initialisations, KMeansRun after 1 and 3 iterations and
# to convergence (plain and alternate), KMeansAssign, QuickAssign and SelectPatch.
if __name__ == "__main__" and "--kmeans" in sys.argv:
    _treecorr.SetOMPThreads(1)
    from cases_km import KM_CASES, KM_MAX_ITER, KM_SEED, KM_TOL, km_inputs, km_spec
    for name in KM_CASES:
        s = km_spec(name)
        cat = km_inputs(name)
        empty = np.array([])
        z = cat["z"] if cat["z"] is not None else empty
        cls = getattr(_treecorr, "NField" + COORDS[s["coords"]])
        fld = cls(cat["x"], cat["y"], z, cat["w"], empty, 0., np.inf, _treecorr.Mean, 0, False,
                  s["min_top"], s["max_top"])
        npatch = s["npatch"]
        dim = 2 if s["coords"] == "flat" else 3
        out = {"x": cat["x"], "y": cat["y"], "w": cat["w"], "ntop": fld.getNTopLevel()}
        if cat["z"] is not None:
            out["z"] = cat["z"]
        for tag, meth in (("tree", fld.KMeansInitTree), ("rand", fld.KMeansInitRand),
                          ("kmpp", fld.KMeansInitKMPP)):
            c = np.zeros((npatch, dim))
            meth(c, npatch, KM_SEED)
            out["init_" + tag] = c
        for tag, iters, alt in (("it1", 1, False), ("it3", 3, False), ("run", KM_MAX_ITER, False),
                                ("alt_it1", 1, True), ("alt_it3", 3, True),
                                ("alt_run", KM_MAX_ITER, True)):
            c = out["init_tree"].copy()
            fld.KMeansRun(c, npatch, iters, KM_TOL, alt)
            out[tag] = c
        pat = np.zeros(s["n"], dtype=int)
        fld.KMeansAssign(out["run"], npatch, pat)
        out["assign"] = pat
        pat = np.zeros(s["n"], dtype=int)
        fld.KMeansAssign(out["alt_run"], npatch, pat)
        out["alt_assign"] = pat
        q = np.zeros(s["n"], dtype=int)
        _treecorr.QuickAssign(out["run"], npatch, cat["x"], cat["y"], z, q)
        out["quick"] = q
        for pp in (0, npatch - 1):
            use = np.zeros(s["n"], dtype=int)
            _treecorr.SelectPatch(pp, out["run"], npatch, cat["x"], cat["y"], z, use)
            out["select_%d" % pp] = use
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(f"{name:16s} ntop={out['ntop']} patches used={len(np.unique(out['assign']))}")


# NNN LogMultipole (the reference's NNNCorr, src/Corr3.cpp:4237) on the catalogs of two GGG
# cases: weight, weight_im, ntri and the mean distances (NNN has no zeta).
if __name__ == "__main__" and "--mp-nnn" in sys.argv:
    _treecorr.SetOMPThreads(1)
    from cases3 import make_inputs3, spec3
    for gname, name in (("ggg_flat_mp", "nnn_flat_mp"), ("ggg_sphere_mp", "nnn_sphere_mp")):
        s = spec3(gname)
        cat = make_inputs3(gname)
        if s["metric"] == "Euclidean":
            b1 = min(s["a"], s["b"])
            min_size, max_size = 2 * s["min_sep"] * b1 / (2. + 3 * b1), s["max_sep"] * b1
        else:
            min_size, max_size = 0.0, 0.0
        nb, mn = s["nbins"], s["max_n"]
        shape = (nb, nb, 2 * mn + 1)
        keys = ("meand1", "meanlogd1", "meand2", "meanlogd2", "meand3", "meanlogd3", "meanu",
                "meanv", "weight", "weight_im", "ntri")
        out = {k: np.zeros(shape) for k in keys}
        e = np.array([])
        corr = _treecorr.NNNCorr(
            _treecorr.LogMultipole, s["min_sep"], s["max_sep"], nb, s["bin_size"], s["b"], s["a"],
            0., 0., mn, 0., 0., 0., 0., 0, 0., 0.,
            -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
            e, e, e, e, e, e, e, e, *[out[k] for k in keys])
        f = build_field("N", s["coords"], cat, min_size, max_size, "mean", False, 3, 10)
        corr.processAuto(f, False, False, METRIC[s["metric"]])
        save = dict(min_size=min_size, max_size=max_size, case=gname)
        for k, v in cat.items():
            if v is not None:
                save["c1_" + k] = v
        for k, v in out.items():
            save["ref_" + k] = v
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **save)
        print(f"{name:16s} ntri={out['ntri'].sum():.6g} weight={out['weight'].sum():.6g}")


# KKK LogMultipole (the reference's KKKCorr, src/Corr3.cpp:4238): zeta (real, imaginary),
# weight, ntri and the mean distances, on the catalogs of two GGG cases with their k column.
if __name__ == "__main__" and "--mp-kkk" in sys.argv:
    _treecorr.SetOMPThreads(1)
    from cases3 import make_inputs3, spec3
    for gname, name in (("ggg_flat_mp", "kkk_flat_mp"), ("ggg_sphere_mp", "kkk_sphere_mp")):
        s = spec3(gname)
        cat = make_inputs3(gname)
        if s["metric"] == "Euclidean":
            b1 = min(s["a"], s["b"])
            min_size, max_size = 2 * s["min_sep"] * b1 / (2. + 3 * b1), s["max_sep"] * b1
        else:
            min_size, max_size = 0.0, 0.0
        nb, mn = s["nbins"], s["max_n"]
        shape = (nb, nb, 2 * mn + 1)
        keys = ("zeta", "zeta_im", "meand1", "meanlogd1", "meand2", "meanlogd2", "meand3",
                "meanlogd3", "meanu", "meanv", "weight", "weight_im", "ntri")
        out = {k: np.zeros(shape) for k in keys}
        e = np.array([])
        corr = _treecorr.KKKCorr(
            _treecorr.LogMultipole, s["min_sep"], s["max_sep"], nb, s["bin_size"], s["b"], s["a"],
            0., 0., mn, 0., 0., 0., 0., 0, 0., 0.,
            -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
            out["zeta"], out["zeta_im"], e, e, e, e, e, e, *[out[k] for k in keys[2:]])
        f = build_field("K", s["coords"], cat, min_size, max_size, "mean", False, 3, 10)
        corr.processAuto(f, False, False, METRIC[s["metric"]])
        save = dict(min_size=min_size, max_size=max_size, case=gname)
        for k, v in cat.items():
            if v is not None:
                save["c1_" + k] = v
        for k, v in out.items():
            save["ref_" + k] = v
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **save)
        print(f"{name:16s} ntri={out['ntri'].sum():.6g} zeta={out['zeta'].sum():.6g}")


# 3-point cross12 with LogMultipole (processCross12 with ordered = 1, src/Corr3.cpp:4199,
# 3730-3768, 1177-1237): vertex 1 from the case's catalog, vertices 2 and 3 from a second
# catalog (seed + 1000), for GGG, NNN, KKK, NKK, KNN, NGG, KGG, GNN and GKK.
X12_CASES = {
    "ggg_flat_mp_x12": ("GGG", "ggg_flat_mp"),
    "ggg_sphere_mp_x12": ("GGG", "ggg_sphere_mp"),
    "nnn_flat_mp_x12": ("NNN", "ggg_flat_mp"),
    "kkk_sphere_mp_x12": ("KKK", "ggg_sphere_mp"),
    "nkk_flat_mp_x12": ("NKK", "ggg_flat_mp"),
    "knn_sphere_mp_x12": ("KNN", "ggg_sphere_mp"),
    "ngg_flat_mp_x12": ("NGG", "ggg_flat_mp"),
    "ngg_sphere_mp_x12": ("NGG", "ggg_sphere_mp"),
    "kgg_sphere_mp_x12": ("KGG", "ggg_sphere_mp"),
    "gnn_flat_mp_x12": ("GNN", "ggg_flat_mp"),
    "gnn_sphere_mp_x12": ("GNN", "ggg_sphere_mp"),
    "gkk_sphere_mp_x12": ("GKK", "ggg_sphere_mp"),
}

if __name__ == "__main__" and "--mp-x12" in sys.argv:
    _treecorr.SetOMPThreads(1)
    from cases3 import make_inputs3, spec3
    only = [a for a in sys.argv[1:] if not a.startswith("--")]
    for name, (letters, gname) in X12_CASES.items():
        if only and name not in only:
            continue
        s = spec3(gname)
        cat1 = make_inputs3(gname)
        cat2 = make_inputs3(gname, seed=20240601 + 1000)
        if s["metric"] == "Euclidean":
            b1 = min(s["a"], s["b"])
            min_size, max_size = 2 * s["min_sep"] * b1 / (2. + 3 * b1), s["max_sep"] * b1
        else:
            min_size, max_size = 0.0, 0.0
        nb, mn = s["nbins"], s["max_n"]
        shape = (nb, nb, 2 * mn + 1)
        common = ("meand1", "meanlogd1", "meand2", "meanlogd2", "meand3", "meanlogd3", "meanu",
                  "meanv", "weight", "weight_im", "ntri")
        zk = (("gam0r", "gam0i", "gam1r", "gam1i", "gam2r", "gam2i", "gam3r", "gam3i")
              if letters == "GGG" else ("gam0r", "gam0i", "gam1r", "gam1i")
              if letters[1:] == "GG" else ("zeta", "zeta_im")
              if ("K" in letters or letters[0] == "G") else ())
        out = {k: np.zeros(shape) for k in zk + common}
        e = np.array([])
        zeta = [out[k] for k in zk] + [e] * (8 - len(zk))
        cls = getattr(_treecorr, letters + "Corr")
        corr = cls(_treecorr.LogMultipole, s["min_sep"], s["max_sep"], nb, s["bin_size"], s["b"],
                   s["a"], 0., 0., mn, 0., 0., 0., 0., 0, 0., 0.,
                   -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
                   *zeta, *[out[k] for k in common])
        f1 = build_field(letters[0], s["coords"], cat1, min_size, max_size, "mean", False, 3, 10)
        f2 = build_field(letters[1], s["coords"], cat2, min_size, max_size, "mean", False, 3, 10)
        corr.processCross12(f1, f2, 1, False, False, METRIC[s["metric"]])
        save = dict(min_size=min_size, max_size=max_size, case=gname, letters=letters)
        for tag, cat in (("c1_", cat1), ("c2_", cat2)):
            for k, v in cat.items():
                if v is not None:
                    save[tag + k] = v
        for k, v in out.items():
            save["ref_" + k] = v
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **save)
        print(f"{name:20s} ntri={out['ntri'].sum():.6g} weight={out['weight'].sum():.6g}")


# The three-field LogMultipole (src/Corr3.cpp:1239-1305) through the reference's
# processCross (3938-3976), processCross21 (3831-3868) and processCross12 with ordered = 0
# (3730-3768): name -> (class, catalogs' case, call, ordered).  Catalogs: the case's, seed +
# 1000 and seed + 2000; a 21 / 12 call takes the first two.
def zeta_keys(letters):
    """The zeta arrays of a 3-point class (ZetaData<0..4>, include/Corr3.h:581-720)."""
    nG = letters.count("G")
    if nG == 3:
        return ("gam0r", "gam0i", "gam1r", "gam1i", "gam2r", "gam2i", "gam3r", "gam3i")
    if letters == "NNN":
        return ()
    if nG == 2:
        return ("gam0r", "gam0i", "gam1r", "gam1i")
    return ("zeta", "zeta_im")


X3_CASES = {
    "ggg_flat_mp_x3o4": ("GGG", "ggg_flat_mp", "cross", 4),
    "ggg_sphere_mp_x3o1": ("GGG", "ggg_sphere_mp", "cross", 1),
    "ggg_flat_mp_x21o3": ("GGG", "ggg_flat_mp", "cross21", 3),
    "kkk_flat_mp_x3o0": ("KKK", "ggg_flat_mp", "cross", 0),
    "nnn_sphere_mp_x12o0": ("NNN", "ggg_sphere_mp", "cross12", 0),
    "ngg_flat_mp_x3o4": ("NGG", "ggg_flat_mp", "cross", 4),
    "gkk_sphere_mp_x3o1": ("GKK", "ggg_sphere_mp", "cross", 1),
    "nnk_flat_mp_x21o3": ("NNK", "ggg_flat_mp", "cross21", 3),
    "nkn_sphere_mp_x3o4": ("NKN", "ggg_sphere_mp", "cross", 4),
    "knk_flat_mp_x3o4": ("KNK", "ggg_flat_mp", "cross", 4),
    "kkn_sphere_mp_x21o3": ("KKN", "ggg_sphere_mp", "cross21", 3),
    "nng_flat_mp_x21o3": ("NNG", "ggg_flat_mp", "cross21", 3),
    "ngn_sphere_mp_x3o4": ("NGN", "ggg_sphere_mp", "cross", 4),
    "kkg_sphere_mp_x21o3": ("KKG", "ggg_sphere_mp", "cross21", 3),
    "kgk_flat_mp_x3o4": ("KGK", "ggg_flat_mp", "cross", 4),
    "gng_flat_mp_x3o4": ("GNG", "ggg_flat_mp", "cross", 4),
    "ggn_sphere_mp_x21o3": ("GGN", "ggg_sphere_mp", "cross21", 3),
    "gkg_sphere_mp_x3o4": ("GKG", "ggg_sphere_mp", "cross", 4),
    "ggk_flat_mp_x21o3": ("GGK", "ggg_flat_mp", "cross21", 3),
    "ggg_flat_mp_x3o2": ("GGG", "ggg_flat_mp", "cross", 2),
    "nnn_flat_mp_x3o3": ("NNN", "ggg_flat_mp", "cross", 3),
    "kkk_sphere_mp_x21o0": ("KKK", "ggg_sphere_mp", "cross21", 0),
}

if __name__ == "__main__" and "--mp-x3" in sys.argv:
    _treecorr.SetOMPThreads(1)
    from cases3 import make_inputs3, spec3
    only = [a for a in sys.argv[1:] if not a.startswith("--")]
    for name, (letters, gname, call, ordered) in X3_CASES.items():
        if only and name not in only:
            continue
        s = spec3(gname)
        cats = [make_inputs3(gname, seed=20240601 + 1000 * i) for i in range(3)]
        cats[0] = make_inputs3(gname)
        if s["metric"] == "Euclidean":
            b1 = min(s["a"], s["b"])
            min_size, max_size = 2 * s["min_sep"] * b1 / (2. + 3 * b1), s["max_sep"] * b1
        else:
            min_size, max_size = 0.0, 0.0
        nb, mn = s["nbins"], s["max_n"]
        shape = (nb, nb, 2 * mn + 1)
        common = ("meand1", "meanlogd1", "meand2", "meanlogd2", "meand3", "meanlogd3", "meanu",
                  "meanv", "weight", "weight_im", "ntri")
        zk = zeta_keys(letters)
        out = {k: np.zeros(shape) for k in zk + common}
        e = np.array([])
        zeta = [out[k] for k in zk] + [e] * (8 - len(zk))
        cls = getattr(_treecorr, letters + "Corr")
        corr = cls(_treecorr.LogMultipole, s["min_sep"], s["max_sep"], nb, s["bin_size"], s["b"],
                   s["a"], 0., 0., mn, 0., 0., 0., 0., 0, 0., 0.,
                   -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
                   *zeta, *[out[k] for k in common])
        kinds = {"cross": letters, "cross21": letters[0] + letters[2], "cross12": letters[:2]}[call]
        fs = [build_field(L, s["coords"], c, min_size, max_size, "mean", False, 3, 10)
              for L, c in zip(kinds, cats)]
        m = METRIC[s["metric"]]
        if call == "cross":
            corr.processCross(fs[0], fs[1], fs[2], ordered, False, False, m)
        elif call == "cross21":
            corr.processCross21(fs[0], fs[1], ordered, False, False, m)
        else:
            corr.processCross12(fs[0], fs[1], ordered, False, False, m)
        save = dict(min_size=min_size, max_size=max_size, case=gname, letters=letters,
                    call=call, ordered=ordered)
        for i in range(len(kinds)):
            for k, v in cats[i].items():
                if v is not None:
                    save[f"c{i + 1}_" + k] = v
        for k, v in out.items():
            save["ref_" + k] = v
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **save)
        print(f"{name:22s} ntri={out['ntri'].sum():.6g} weight={out['weight'].sum():.6g}")


# The benchmark configurations' own shapes and binnings (tests/golden/cases_bench.py): the
# catalogs are regenerated bit-identically from their seeds, so only the outputs and a hash
# of the inputs are stored.
def run_bench2(name):
    from cases_bench import bench2_inputs, bench2_spec, catalog_hash
    s = bench2_spec(name)
    cat = bench2_inputs(name)
    B = s["bins"]
    nb = B["nbins"]
    out = {k: np.zeros(nb) for k in ("xi0", "xi1", "xi2", "xi3", "meanr", "meanlogr",
                                      "weight", "npairs")}
    corr = _treecorr.GGCorr(
        _treecorr.Log, B["min_sep"], B["max_sep"], nb, B["bin_size"], B["b"], B["a"],
        -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
        out["xi0"], out["xi1"], out["xi2"], out["xi3"], out["meanr"], out["meanlogr"],
        out["weight"], out["npairs"])
    f = build_field("G", s["coords"], cat, s["min_size"], s["max_size"], s["split"],
                    s["brute"], s["min_top"], s["max_top"])
    corr.processAuto(f, False, False, METRIC[s["metric"]])
    save = dict(min_size=s["min_size"], max_size=s["max_size"], ntop=f.getNTopLevel(),
                input_sha256=catalog_hash(cat))
    for k, v in out.items():
        save["ref_" + k] = v
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **save)
    return out


def run_bench3(name):
    from cases_bench import bench3_inputs, bench3_spec, catalog_hash
    s = bench3_spec(name)
    cat = bench3_inputs(name)
    nb, mn = s["nbins"], s["max_n"]
    shape = (nb, nb, 2 * mn + 1)
    keys = ("gam0r", "gam0i", "gam1r", "gam1i", "gam2r", "gam2i", "gam3r", "gam3i",
            "meand1", "meanlogd1", "meand2", "meanlogd2", "meand3", "meanlogd3", "meanu",
            "meanv", "weight", "weight_im", "ntri")
    out = {k: np.zeros(shape) for k in keys}
    corr = _treecorr.GGGCorr(
        _treecorr.LogMultipole, s["min_sep"], s["max_sep"], nb, s["bin_size"], s["b"], s["a"],
        0., 0., mn, 0., 0., 0., 0., 0, 0., 0.,
        -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
        *[out[k] for k in keys])
    f = build_field("G", s["coords"], cat, s["min_size"], s["max_size"], "mean", False, 3, 10)
    corr.processAuto(f, False, False, METRIC[s["metric"]])
    save = dict(min_size=s["min_size"], max_size=s["max_size"], input_sha256=catalog_hash(cat))
    for k, v in out.items():
        save["ref_" + k] = v
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **save)
    return out


if __name__ == "__main__" and "--bench" in sys.argv:
    import time
    from cases_bench import BENCH2, BENCH3
    _treecorr.SetOMPThreads(1)
    only = [a for a in sys.argv[1:] if not a.startswith("--")]
    for name in BENCH2:
        if only and name not in only:
            continue
        t0 = time.time()
        out = run_bench2(name)
        print(f"{name:16s} npairs={out['npairs'].sum():.0f} weight={out['weight'].sum():.6g} "
              f"({time.time() - t0:.1f} s)", flush=True)
    for name in BENCH3:
        if only and name not in only:
            continue
        t0 = time.time()
        out = run_bench3(name)
        print(f"{name:16s} ntri={out['ntri'].sum():.6g} weight={out['weight'].sum():.6g} "
              f"({time.time() - t0:.1f} s)", flush=True)
