"""The `_treecorr` call logs of TreeCorr's own Python layer (tests/golden/api_*.npz, made by
tests/golden/make_api_trace.py with the reference's compiled module) and their replay.

A log holds every boundary call the Python layer made while a scenario ran through the
public API (Catalog, the Correlation classes, process, jackknife covariance, toSAS): class
constructions ("new"), method calls on the constructed objects ("call") and module functions
("fn"), with their arguments, the state of the aliased output arrays before and after each
call (the Python layer reads and clears them between calls), the array arguments after the
call, the return value, and the scenario's final Python-level results ("final_*").
"""
import json
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCENARIOS = ("gg_flat", "gg_sphere_jk", "nn_ls", "kk_exact", "ggg_mp")
# Functions whose return value is a machine property, not a result.
UNCOMPARED = {"SetOMPThreads", "GetOMPThreads"}


class Trace:
    def __init__(self, name):
        g = np.load(os.path.join(HERE, "api_%s.npz" % name))
        self.name = name
        self.events = json.loads(str(g["events"]))
        self.arrays = {int(k[1:]): g[k] for k in g.files if k.startswith("a") and k[1:].isdigit()}
        self.final = {k: g["final_" + k] for k in json.loads(str(g["final_keys"]))}

    def arr(self, ref):
        return self.arrays[ref["arr"]].copy()


def decode(T, tr, v, objs):
    """An argument of the log as a value for module T (objects: T's replayed objects)."""
    if isinstance(v, dict):
        if "obj" in v:
            return objs[v["obj"]]
        if "arr" in v:
            return tr.arr(v)
        if "enum" in v:
            return getattr(T, v["name"])
    if isinstance(v, list):
        return [decode(T, tr, x, objs) for x in v]
    return v


def close(got, ref, key, rtol):
    """Max |got - ref| relative to the scale of ref (exact for integer-valued counts)."""
    got, ref = np.asarray(got, dtype=float), np.asarray(ref, dtype=float)
    if got.shape != ref.shape:
        return f"{key}: shape {got.shape} != {ref.shape}"
    if key == "npairs" or key == "ntri":
        return None if np.array_equal(got, ref) else f"{key}: counts differ"
    scale = np.abs(ref).max() if ref.size else 0.
    if scale == 0.:
        return None if not np.abs(got).any() else f"{key}: nonzero where the reference is 0"
    err = np.abs(got - ref).max() / scale
    return None if err <= rtol else f"{key}: {err:.2e} > {rtol:g}"


def replay(T, tr, rtol=1e-5, out_names=None):
    """Replays the log against module T: every call with the logged arguments, the output
    arrays set to their logged state before the call.  Returns (problems, increments), where
    increments[i] are the output arrays' changes by call event i of a correlation object."""
    objs, outs, problems, incs = {}, {}, [], {}
    for i, e in enumerate(tr.events):
        if e["op"] == "new":
            args = [decode(T, tr, a, objs) for a in e["args"]]
            objs[e["id"]] = getattr(T, e["cls"])(*args)
            outs[e["id"]] = [a for a in args if isinstance(a, np.ndarray)]
            continue
        if e["op"] == "fn":
            args = [decode(T, tr, a, objs) for a in e["args"]]
            ret = getattr(T, e["name"])(*args)
            what = e["name"]
        else:
            obj = objs[e["id"]]
            for a, ref in zip(outs[e["id"]], e["outs_before"]):
                a[...] = tr.arr(ref)
            args = [decode(T, tr, a, objs) for a in e["args"]]
            ret = getattr(obj, e["method"])(*args)
            what = "%s#%d.%s" % (e.get("cls", ""), e["id"], e["method"])
            names = (out_names or {}).get(e["id"])
            arrays = outs[e["id"]]
            for k, (a, ref) in enumerate(zip(arrays, e["outs"])):
                key = names[k] if names else "out%d" % k
                msg = close(a, tr.arr(ref), key, rtol)
                if msg:
                    problems.append(f"event {i} {what}: {msg}")
            if arrays:
                incs[i] = [a - tr.arr(b) for a, b in zip(arrays, e["outs_before"])]
        for k, (a, ref) in enumerate(zip(args, e["after"])):
            if ref is not None and isinstance(a, np.ndarray):
                msg = close(a, tr.arr(ref), "arg%d" % k, rtol)
                if msg:
                    problems.append(f"event {i} {what}: {msg}")
        name = e.get("name") or e.get("method")
        if name not in UNCOMPARED and e["ret"] is not None and not isinstance(e["ret"], dict):
            if isinstance(e["ret"], float):
                if abs(ret - e["ret"]) > rtol * max(abs(e["ret"]), 1e-300):
                    problems.append(f"event {i} {what}: returned {ret} != {e['ret']}")
            elif ret != e["ret"]:
                problems.append(f"event {i} {what}: returned {ret} != {e['ret']}")
    return problems, incs


def corr2_out_names(tr):
    """The output array names of each 2-point correlation object of a log, in the order of
    the reference's constructor (xi0..xi3 where present, meanr, meanlogr, weight, npairs)."""
    names = {}
    for e in tr.events:
        if e["op"] == "new" and e["cls"].endswith("Corr") and len(e["args"]) == 20:
            present = [isinstance(a, dict) and "arr" in a for a in e["args"][12:20]]
            keys = ["xi0", "xi1", "xi2", "xi3", "meanr", "meanlogr", "weight", "npairs"]
            names[e["id"]] = [k for k, p in zip(keys, present) if p]
    return names


def final_outs(tr):
    """The last logged output arrays of each 2-point correlation object of a log."""
    corrs = corr2_out_names(tr)
    last = {}
    for e in tr.events:
        if e["op"] == "call" and e["id"] in corrs:
            last[e["id"]] = [tr.arr(r) for r in e["outs"]]
    return last


def patch_pairs(tr, incs=None):
    """Per-patch-pair results of the jackknife scenario: for every process call of the
    GGCorr, (i, j) of its patch fields and the increment it added ([8, nbins]: weight, meanr,
    meanlogr, xi0..xi3, npairs).  Patch fields are told apart by their points: the field's x
    column equals the catalog's x (from GenerateXYZ) at the points of one patch."""
    ev = tr.events
    xyz = next(e for e in ev if e["op"] == "fn" and e["name"] == "GenerateXYZ")
    xall = tr.arr(xyz["after"][0])
    patch = tr.final["patch"]
    field_patch = {}
    for e in ev:
        if e["op"] == "new" and e["cls"].startswith("GField"):
            x = tr.arr(e["args"][0])
            for p in range(int(patch.max()) + 1):
                xp = xall[patch == p]
                if len(xp) == len(x) and np.array_equal(xp, x):
                    field_patch[e["id"]] = p
    gid = next(e["id"] for e in ev if e["op"] == "new" and e["cls"] == "GGCorr")
    pairs, res = [], []
    for i, e in enumerate(ev):
        if e["op"] != "call" or e["id"] != gid or not e["method"].startswith("process"):
            continue
        f = [a["obj"] for a in e["args"] if isinstance(a, dict) and "obj" in a]
        pi = field_patch[f[0]]
        pj = field_patch[f[1]] if len(f) > 1 else pi
        inc = incs[i] if incs is not None else [tr.arr(a) - tr.arr(b)
                                                for a, b in zip(e["outs"], e["outs_before"])]
        xi0, xi1, xi2, xi3, meanr, meanlogr, weight, npairs = inc
        pairs.append((pi, pj))
        res.append(np.stack([weight, meanr, meanlogr, xi0, xi1, xi2, xi3, npairs]))
    return pairs, np.array(res)


def finalize_xi(xi, weight):
    """The reference's _finalize for the xi arrays (treecorr/corr2base.py:1274-1279)."""
    out = np.zeros_like(xi)
    m = weight != 0
    out[m] = xi[m] / weight[m]
    return out
