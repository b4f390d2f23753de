"""Fixtures of TreeCorr's catalog ingestion (Catalog._finish_input, treecorr/catalog.py:
1343-1487): the flag -> weight conversion, the NaN checks, the wpos == 0 rule, sumw and the
removal of zero-weight rows, made by the reference's own Python Catalog.

Run where the reference sources are (not on the GPU machine):

    make -f oracle/Makefile.ref -j8 REF=$TREECORR_REFERENCE
    TREECORR_REFERENCE=/path/to/TreeCorr python tests/golden/make_catalog_golden.py

It imports TreeCorr's Python package from the reference tree with the test-only `coord`
stand-in (tests/golden/coord_shim) and the reference's compiled module (oracle/_ref), builds
each catalog below from arrays, and stores the input columns, the configuration and the
catalog's columns, sumw, ntot, nobj and _get_center_size() (the centre and size that the
patch loops' triviallyZero tests use) after construction in tests/golden/catalog_<name>.npz.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_api_trace import load_reference_module  # noqa: E402

COLS = ("x", "y", "z", "ra", "dec", "r", "k", "g1", "g2", "w", "wpos")


def _nan_rows(rng, a, m):
    a = a.copy()
    a[rng.choice(len(a), m, replace=False)] = np.nan
    return a


def cases():
    rng = np.random.default_rng(20261204)
    n = 3000
    out = {}
    # Flat catalog with flags (ok_flag 1: any other bit removes the row), NaNs in four
    # columns including w, and some zero weights.
    w = rng.uniform(0.5, 1.5, n)
    w[rng.choice(n, 40, replace=False)] = 0.
    out["flat_flags_nan"] = (dict(
        x=_nan_rows(rng, rng.uniform(0, 100, n), 5), y=rng.uniform(0, 100, n),
        k=_nan_rows(rng, rng.normal(0, 0.02, n), 3),
        g1=_nan_rows(rng, rng.normal(0, 0.2, n), 7), g2=rng.normal(0, 0.2, n),
        w=_nan_rows(rng, w, 4), flag=rng.integers(0, 8, n)), dict(ok_flag=1))
    # Flat catalog with wpos: zero wpos on some rows (some with w != 0), NaN in wpos.
    wpos = rng.uniform(0.5, 1.5, n)
    wpos[rng.choice(n, 30, replace=False)] = 0.
    w2 = rng.uniform(0.5, 1.5, n)
    out["flat_wpos"] = (dict(x=rng.uniform(0, 50, n), y=rng.uniform(0, 50, n),
                             k=rng.normal(0, 0.02, n), w=w2, wpos=_nan_rows(rng, wpos, 2)),
                        dict())
    # 3-d catalog with an ignore_flag and no weights, keeping the zero-weight rows.
    out["3d_keep"] = (dict(x=rng.uniform(0, 10, n), y=rng.uniform(0, 10, n),
                           z=_nan_rows(rng, rng.uniform(0, 10, n), 6),
                           g1=rng.normal(0, 0.2, n), g2=rng.normal(0, 0.2, n),
                           flag=rng.integers(0, 8, n)),
                      dict(ignore_flag=4, keep_zero_weight=True))
    # Sky catalog (ra, dec, r in radians) with NaNs in dec and r and weights.
    out["sky_radec"] = (dict(ra=rng.uniform(0, 0.5, n),
                             dec=_nan_rows(rng, rng.uniform(-0.3, 0.3, n), 4),
                             r=_nan_rows(rng, rng.uniform(100, 200, n), 3),
                             g1=rng.normal(0, 0.2, n), g2=rng.normal(0, 0.2, n),
                             w=rng.uniform(0.5, 1.5, n)),
                        dict(ra_units="rad", dec_units="rad"))
    # No weights, NaN in k: the NaN rows get w = 0 and are removed.
    out["no_w_nan"] = (dict(x=rng.uniform(0, 10, n), y=rng.uniform(0, 10, n),
                            k=_nan_rows(rng, rng.normal(0, 0.02, n), 9)), dict())
    # Nothing to do: w stays trivial, sumw = ntot.
    out["trivial"] = (dict(x=rng.uniform(0, 10, n), y=rng.uniform(0, 10, n),
                           g1=rng.normal(0, 0.2, n), g2=rng.normal(0, 0.2, n)), dict())
    return out


def main():
    ref_root = os.environ.get("TREECORR_REFERENCE")
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "treecorr")):
        sys.exit("set TREECORR_REFERENCE to the TreeCorr source tree")
    sys.modules["treecorr._treecorr"] = load_reference_module()
    sys.path.insert(0, os.path.join(HERE, "coord_shim"))
    sys.path.insert(0, ref_root)
    import treecorr
    for name, (cols, cfg) in cases().items():
        cat = treecorr.Catalog(**{k: v.copy() for k, v in cols.items()}, **cfg)
        save = {"config": np.array(json.dumps(cfg))}
        for k, v in cols.items():
            save["in_" + k] = v
        for k in COLS:
            v = getattr(cat, k)
            if v is not None:
                save["out_" + k] = np.asarray(v)
        save["sumw"] = np.float64(cat.sumw)
        save["ntot"] = np.int64(cat.ntot)
        save["nobj"] = np.int64(cat.nobj)
        save["nontrivial_w"] = np.bool_(cat.nontrivial_w)
        save["center_size"] = np.array(cat._get_center_size(), dtype=float)
        np.savez_compressed(os.path.join(HERE, "catalog_%s.npz" % name), **save)
        print(f"{name:16s} ntot {cat.ntot} nobj {cat.nobj} sumw {cat.sumw:.6f} "
              f"nontrivial {cat.nontrivial_w}")


if __name__ == "__main__":
    main()
