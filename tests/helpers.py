"""Shared helpers of the tests: golden cases, the GPU path through the _treecorr mirror,
and the oracle (the checker)."""
import sys

import numpy as np

from cases import CASES, kinds, spec_dict, xi_count  # noqa: F401  (tests/golden on sys.path)

OUT_KEYS = ("xi0", "xi1", "xi2", "xi3", "meanr", "meanlogr", "weight", "npairs")
COORD_NAME = {"flat": "Flat", "spherical": "Sphere", "3d": "ThreeD"}


def load_case(name):
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    g = np.load(os.path.join(here, name + ".npz"))
    s = spec_dict(name)
    c1 = {k[3:]: g[k] for k in g.files if k.startswith("c1_")}
    c2 = {k[3:]: g[k] for k in g.files if k.startswith("c2_")} if s["n2"] else None
    bins = dict(min_sep=s["min_sep"], max_sep=s["max_sep"], nbins=s["nbins"],
                bin_size=float(g["bin_size"]), b=float(g["b"]), a=float(g["a"]))
    ref = {k: g["ref_" + k] for k in OUT_KEYS}
    return s, c1, c2, bins, float(g["min_size"]), float(g["max_size"]), ref


def field_args(dtype, cat):
    if dtype in "ZVGTQ":
        return [cat["g1"], cat["g2"]]
    if dtype == "K":
        return [cat["k"]]
    return []


def gpu_field(T, dtype, coords, cat, min_size, max_size, split="mean", brute=False,
              min_top=3, max_top=10):
    cls = getattr(T, dtype + "Field" + COORD_NAME[coords])
    sm = {"mean": T.Mean, "median": T.Median, "middle": T.Middle}[split]
    e = np.array([])
    z = cat.get("z") if cat.get("z") is not None else e
    return cls(cat["x"], cat["y"], z, *field_args(dtype, cat), cat["w"], e, min_size,
               max_size, sm, 0, brute, min_top, max_top)


def gpu_process(T, dtype, metric, bins, f1, f2=None, quick=False):
    """dtype: "G" (GG) or a pair such as "NG"; the class is d1 + d2 + "Corr"."""
    nb = bins["nbins"]
    out = {k: np.zeros(nb) for k in OUT_KEYS}
    e = np.array([])
    nxi = xi_count(dtype)
    xi = [out["xi%d" % i] if i < nxi else e for i in range(4)]
    d1, d2 = kinds(dtype)
    corr = getattr(T, d1 + d2 + "Corr")(T.Log, bins["min_sep"], bins["max_sep"], nb,
                                          bins["bin_size"], bins["b"], bins["a"],
                                          -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
                                          *xi, out["meanr"], out["meanlogr"], out["weight"],
                                          out["npairs"])
    m = T.Euclidean if metric == "Euclidean" else T.Arc
    if f2 is None:
        corr.processAuto(f1, False, quick, m)
    else:
        corr.processCross(f1, f2, False, quick, m)
    out["_stats"] = corr.stats()
    return out


def oracle_field(dtype, coords, cat, min_size, max_size, split="mean", brute=False,
                 min_top=3, max_top=10):
    from oracle import oracle as O
    d = field_args(dtype, cat) + [None, None]
    return O.OracleField(dtype, coords, cat["x"], cat["y"], cat.get("z"), d[0], d[1], cat["w"],
                         None, min_size, max_size, split, brute, min_top, max_top)


def oracle_process(dtype, metric, bins, f1, f2=None, quick=False, nthreads=0):
    from oracle import oracle as O
    return O.process(dtype, metric, bins, f1, f2, quick=quick, nthreads=nthreads)


def assert_outputs_close(got, ref, dtype, rtol=1e-5, exact_npairs=True, label=""):
    """npairs bit-identical; weight/meanr/meanlogr/xi within rtol of the array's scale."""
    if exact_npairs:
        assert np.array_equal(got["npairs"], ref["npairs"]), \
            f"{label} npairs differ: {got['npairs'] - ref['npairs']}"
    keys = ["weight", "meanr", "meanlogr"] + ["xi%d" % i for i in range(xi_count(dtype))]
    for k in keys:
        r = np.asarray(ref[k])
        g = np.asarray(got[k])
        scale = np.abs(r).max() if r.size else 0.
        if k in ("xi0", "xi1", "xi2", "xi3"):
            # xi values are signed sums; compare against the summed weight scale too, so
            # that bins whose xi is ~0 by cancellation are judged on an absolute scale.
            scale = max(scale, 1e-3 * np.abs(ref["weight"]).max())
        err = np.abs(g - r).max() / max(scale, 1e-300)
        assert err <= rtol, f"{label} {k}: max rel err {err:.3e} > {rtol:g}\n got {g}\n ref {r}"


def case_fields(make, s, c1, c2, min_size, max_size):
    """The case's two fields built by make(dtype, coords, cat, ...) (GPU or oracle); the
    second is None for an auto correlation."""
    d1, d2 = kinds(s["dtype"])
    f1 = make(d1, s["coords"], c1, min_size, max_size, s["split"], s["brute"], s["min_top"],
              s["max_top"])
    f2 = None
    if c2 is not None:
        f2 = make(d2, s["coords"], c2, min_size, max_size, s["split"], s["brute"],
                  s["min_top"], s["max_top"])
    return f1, f2
