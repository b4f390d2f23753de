"""Record what TreeCorr's unchanged Python layer sends across the `_treecorr` boundary.

Run where the reference sources are (not on the GPU machine):

    make -f oracle/Makefile.ref -j8 REF=$TREECORR_REFERENCE
    TREECORR_REFERENCE=/path/to/TreeCorr python tests/golden/make_api_trace.py

It imports TreeCorr's own Python package from the reference tree with the test-only `coord`
stand-in (tests/golden/coord_shim) and with `treecorr._treecorr` replaced by a recording proxy
around the reference's compiled module (oracle/_ref).  Each scenario below drives the public
API as a user would (Catalog, the Correlation classes, process, calculateXi, jackknife
covariances, toSAS).  The proxy logs every constructor, method and function call on the
boundary with its arguments, the contents of the array arguments after the call (the output
arrays the reference aliases and adds into), and the return value.  The scenario's final
Python-level results are stored with the log in tests/golden/api_<scenario>.npz.

tests/test_gpu_api_replay.py replays each log against treecorr_gb300._treecorr -- the same
calls with the same arguments in the same order -- and compares the boundary outputs.
tests/test_api_trace.py checks on the CPU that the module exposes every name and accepts
every call the log holds, and that the oracle's jackknife restatement gives the reference's
covariance from the logged per-patch-pair results.
"""
import glob
import hashlib
import importlib.machinery
import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def load_reference_module():
    so = glob.glob(os.path.join(ROOT, "oracle", "_ref", "_treecorr*.so"))
    if not so:
        sys.exit("reference module not built: make -f oracle/Makefile.ref -j8")
    loader = importlib.machinery.ExtensionFileLoader("_treecorr", so[0])
    spec = importlib.util.spec_from_file_location("_treecorr", so[0], loader=loader)
    mod = importlib.util.module_from_spec(spec)
    loader.exec_module(mod)
    return mod


def is_enum(v):
    return hasattr(type(v), "__members__") and hasattr(v, "name")


class Recorder:
    def __init__(self, mod):
        self.mod = mod
        self.events = []
        self.arrays = []
        self._keys = {}
        self.next_id = 0

    def arr(self, a):
        a = np.ascontiguousarray(a)
        h = hashlib.sha1(a.tobytes()).hexdigest() + str(a.dtype) + str(a.shape)
        if h not in self._keys:
            self._keys[h] = len(self.arrays)
            self.arrays.append(a.copy())
        return {"arr": self._keys[h]}

    def enc(self, v):
        if isinstance(v, Proxy):
            return {"obj": v._pid}
        if isinstance(v, np.ndarray):
            return self.arr(v)
        if is_enum(v):
            return {"enum": type(v).__name__, "name": v.name}
        if isinstance(v, (bool, int, float, str)) or v is None:
            return v
        if isinstance(v, (np.integer,)):
            return int(v)
        if isinstance(v, (np.floating,)):
            return float(v)
        if isinstance(v, (list, tuple)):
            return [self.enc(x) for x in v]
        raise TypeError("cannot record %r" % type(v))


def unwrap(v):
    return v._real if isinstance(v, Proxy) else v


class Proxy:
    """A boundary object (field or correlation) of the reference module, recorded."""

    def __init__(self, rec, real, pid, arrays):
        object.__setattr__(self, "_rec", rec)
        object.__setattr__(self, "_real", real)
        object.__setattr__(self, "_pid", pid)
        object.__setattr__(self, "_arrays", arrays)   # the output arrays it aliases

    def __getattr__(self, name):
        attr = getattr(self._real, name)
        if not callable(attr):
            return attr
        rec = self._rec

        def call(*args):
            before = [rec.enc(a) for a in args]
            # The Python layer also reads and clears the aliased output arrays between calls
            # (outside the boundary): their state before the call is part of its input.
            outs_before = [rec.arr(a) for a in self._arrays]
            ret = attr(*[unwrap(a) for a in args])
            after = [rec.arr(a) if isinstance(a, np.ndarray) else None for a in args]
            outs = [rec.arr(a) for a in self._arrays]
            rec.events.append({"op": "call", "id": self._pid, "method": name, "args": before,
                               "after": after, "outs_before": outs_before, "outs": outs,
                               "ret": rec.enc(ret)})
            return ret
        return call


class Ctor:
    """Stands in for a boundary class.  A callable object, not a function, so that the Python
    layer can keep it as a class attribute (`_builder = _treecorr.GGCorr`) without it being
    bound as a method."""

    def __init__(self, rec, cls, name):
        self.rec, self.cls, self.name = rec, cls, name

    def __call__(self, *args):
        rec = self.rec
        pid = rec.next_id
        rec.next_id += 1
        arrays = [a for a in args if isinstance(a, np.ndarray)]
        rec.events.append({"op": "new", "cls": self.name, "id": pid,
                           "args": [rec.enc(a) for a in args]})
        real = self.cls(*[unwrap(a) for a in args])
        return Proxy(rec, real, pid, arrays)


def make_proxy_module(rec):
    import types
    mod = rec.mod
    px = types.ModuleType("treecorr._treecorr")
    px.__file__ = mod.__file__
    for name in dir(mod):
        if name.startswith("__"):
            continue
        v = getattr(mod, name)
        if isinstance(v, type) and not is_enum_type(v):
            setattr(px, name, Ctor(rec, v, name))
        elif callable(v) and not isinstance(v, type):
            def fn(*args, _f=v, _name=name):
                before = [rec.enc(a) for a in args]
                ret = _f(*[unwrap(a) for a in args])
                after = [rec.arr(a) if isinstance(a, np.ndarray) else None for a in args]
                rec.events.append({"op": "fn", "name": _name, "args": before, "after": after,
                                   "ret": rec.enc(ret)})
                return ret
            setattr(px, name, fn)
        else:
            setattr(px, name, v)
    return px


def is_enum_type(t):
    return hasattr(t, "__members__")


# ----------------------------------------------------------------------------------------
# Scenarios: small catalogs (seconds for the reference), every step through the public API.

def scenario_gg_flat(treecorr):
    rng = np.random.default_rng(31)
    n = 6000
    x, y = rng.uniform(0, 200, n), rng.uniform(0, 200, n)
    g1, g2, w = rng.normal(0, 0.2, n), rng.normal(0, 0.2, n), rng.uniform(0.5, 1.5, n)
    cat = treecorr.Catalog(x=x, y=y, g1=g1, g2=g2, w=w, x_units='arcmin', y_units='arcmin')
    gg = treecorr.GGCorrelation(min_sep=1., max_sep=50., nbins=12, sep_units='arcmin',
                                bin_slop=0.5)
    gg.process(cat)
    return {"xip": gg.xip, "xim": gg.xim, "xip_im": gg.xip_im, "xim_im": gg.xim_im,
            "meanr": gg.meanr, "meanlogr": gg.meanlogr, "npairs": gg.npairs,
            "weight": gg.weight, "varxip": gg.varxip, "varxim": gg.varxim}


def scenario_gg_sphere_jk(treecorr):
    rng = np.random.default_rng(32)
    n = 8000
    ra = rng.uniform(10., 16., n)
    dec = np.degrees(np.arcsin(rng.uniform(np.sin(np.radians(-3.)), np.sin(np.radians(3.)), n)))
    g1, g2, w = rng.normal(0, 0.25, n), rng.normal(0, 0.25, n), rng.uniform(0.5, 1.5, n)
    cat = treecorr.Catalog(ra=ra, dec=dec, g1=g1, g2=g2, w=w, ra_units='deg', dec_units='deg',
                           npatch=6, rng=np.random.default_rng(5))
    gg = treecorr.GGCorrelation(min_sep=2., max_sep=120., nbins=10, sep_units='arcmin',
                                bin_slop=0.2, var_method='jackknife')
    gg.process(cat)
    return {"xip": gg.xip, "xim": gg.xim, "npairs": gg.npairs, "weight": gg.weight,
            "meanr": gg.meanr, "cov": gg.cov, "varxip": gg.varxip,
            "patch": cat.patch.astype(np.int64), "patch_centers": cat.patch_centers}


def scenario_nn_ls(treecorr):
    rng = np.random.default_rng(33)
    n, nr = 5000, 10000
    x, y = rng.uniform(0, 300, n), rng.uniform(0, 300, n)
    rx, ry = rng.uniform(0, 300, nr), rng.uniform(0, 300, nr)
    d = treecorr.Catalog(x=x, y=y)
    r = treecorr.Catalog(x=rx, y=ry)
    kw = dict(min_sep=1., max_sep=60., nbins=10, bin_slop=0.0)
    dd, rr, dr = (treecorr.NNCorrelation(**kw) for _ in range(3))
    dd.process(d)
    rr.process(r)
    dr.process(d, r)
    xi, varxi = dd.calculateXi(rr=rr, dr=dr)
    return {"xi": xi, "varxi": varxi, "dd_npairs": dd.npairs, "rr_npairs": rr.npairs,
            "dr_npairs": dr.npairs}


def scenario_kk_exact(treecorr):
    rng = np.random.default_rng(34)
    n = 6000
    x, y = rng.uniform(0, 150, n), rng.uniform(0, 150, n)
    k, w = rng.normal(0, 0.02, n), rng.uniform(0.5, 1.5, n)
    cat = treecorr.Catalog(x=x, y=y, k=k, w=w)
    kk = treecorr.KKCorrelation(min_sep=1., max_sep=40., nbins=10, bin_slop=0.0,
                                angle_slop=0.0)
    kk.process(cat)
    return {"xi": kk.xi, "varxi": kk.varxi, "npairs": kk.npairs, "weight": kk.weight,
            "meanr": kk.meanr}


def scenario_ggg_mp(treecorr):
    rng = np.random.default_rng(35)
    n = 1500
    x, y = rng.uniform(0, 60, n), rng.uniform(0, 60, n)
    g1, g2, w = rng.normal(0, 0.25, n), rng.normal(0, 0.25, n), rng.uniform(0.5, 1.5, n)
    cat = treecorr.Catalog(x=x, y=y, g1=g1, g2=g2, w=w)
    ggg = treecorr.GGGCorrelation(min_sep=2., max_sep=20., nbins=6, max_n=8,
                                  bin_type='LogMultipole')
    ggg.process(cat)
    out = {"gam0": ggg.gam0, "gam1": ggg.gam1, "gam2": ggg.gam2, "gam3": ggg.gam3,
           "weight": ggg.weight, "ntri": ggg.ntri}
    sas = ggg.toSAS(phi_bin_size=0.3)
    out.update({"sas_gam0": sas.gam0, "sas_gam1": sas.gam1, "sas_gam2": sas.gam2,
                "sas_gam3": sas.gam3, "sas_weight": sas.weight, "sas_phi": sas.phi})
    return out


SCENARIOS = {"gg_flat": scenario_gg_flat, "gg_sphere_jk": scenario_gg_sphere_jk,
             "nn_ls": scenario_nn_ls, "kk_exact": scenario_kk_exact, "ggg_mp": scenario_ggg_mp}


def main():
    ref_root = os.environ.get("TREECORR_REFERENCE")
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "treecorr")):
        sys.exit("set TREECORR_REFERENCE to the TreeCorr source tree")
    mod = load_reference_module()
    mod.SetOMPThreads(1)
    names = sys.argv[1:] or list(SCENARIOS)
    sys.path.insert(0, os.path.join(HERE, "coord_shim"))
    for name in names:
        rec = Recorder(mod)
        for k in [k for k in sys.modules if k == "treecorr" or k.startswith("treecorr.")]:
            del sys.modules[k]
        sys.modules["treecorr._treecorr"] = make_proxy_module(rec)
        sys.path.insert(0, ref_root)
        import treecorr
        sys.path.remove(ref_root)
        final = SCENARIOS[name](treecorr)
        save = {"events": np.array(json.dumps(rec.events)),
                "final_keys": np.array(json.dumps(sorted(final)))}
        for i, a in enumerate(rec.arrays):
            save["a%d" % i] = a
        for k, v in final.items():
            save["final_" + k] = np.asarray(v)
        np.savez_compressed(os.path.join(HERE, "api_%s.npz" % name), **save)
        calls = sorted({e.get("cls") or e.get("method") or e.get("name") for e in rec.events})
        print(f"{name:14s} {len(rec.events)} boundary calls, {len(rec.arrays)} arrays: {calls}")


if __name__ == "__main__":
    main()
