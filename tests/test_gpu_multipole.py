"""GPU parity of the GGG LogMultipole accumulation against the reference's golden outputs
and the oracle."""
import os
import sys

import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu

MP_OUT = ("gam0r", "gam0i", "gam1r", "gam1i", "gam2r", "gam2i", "gam3r", "gam3i",
          "meand1", "meanlogd1", "meand2", "meanlogd2", "meand3", "meanlogd3", "meanu",
          "meanv", "weight", "weight_im", "ntri")


def gpu_multipole(T, s, cat, min_size, max_size):
    nb, mn = s["nbins"], s["max_n"]
    shape = (nb, nb, 2 * mn + 1)
    out = {k: np.zeros(shape) for k in MP_OUT}
    corr = T.GGGCorr(T.LogMultipole, s["min_sep"], s["max_sep"], nb, s["bin_size"], s["b"],
                     s["a"], 0., 0., mn, 0., 0., 0., 0., 0, 0., 0.,
                     -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
                     *[out[k] for k in MP_OUT])
    f = H.gpu_field(T, "G", s["coords"], cat, min_size, max_size)
    m = T.Euclidean if s["metric"] == "Euclidean" else T.Arc
    corr.processAuto(f, False, False, m)
    return out


# G_n / W_n terms, their sums within a warp's run of records, and the products of the
# contraction are FP32; every running sum is FP64.  Bound on max|gpu - ref| / max|ref| per
# output array (the reference's own multipole test uses rtol 1e-4 on gam).
TOL = 1e-5


def max_rel_err(out, ref):
    return {k: np.abs(out[k] - ref[k]).max() / max(np.abs(ref[k]).max(), 1e-300) for k in ref}


@pytest.mark.parametrize("name", ["ggg_flat_mp", "ggg_flat_mp_n20", "ggg_flat_mp_bs0",
                                  "ggg_sphere_mp"])
def test_multipole_golden(gpu_lib, name):
    from cases3 import spec3
    s = spec3(name)
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    cat = {k[3:]: g[k] for k in g.files if k.startswith("c1_")}
    out = gpu_multipole(gpu_lib, s, cat, float(g["min_size"]), float(g["max_size"]))
    assert np.array_equal(out["ntri"], g["ref_ntri"]), name
    err = max_rel_err(out, {k: g["ref_" + k] for k in MP_OUT})
    print(name, " ".join(f"{k}={v:.1e}" for k, v in err.items() if v > 0))
    for k, v in err.items():
        assert v <= TOL, f"{name} {k}: {v:.3e}"


def test_multipole_record_waves(gpu_lib, monkeypatch):
    """A record buffer of a few vertices forces many finish/contract waves and the in-place
    FP64 contraction of records that do not fit; the result must not change."""
    from cases3 import spec3
    name = "ggg_flat_mp"
    s = spec3(name)
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    cat = {k[3:]: g[k] for k in g.files if k.startswith("c1_")}
    base = gpu_multipole(gpu_lib, s, cat, float(g["min_size"]), float(g["max_size"]))
    monkeypatch.setenv("TCGPU_MP_RECORD_BYTES", str(40 * 16 * 1024))
    small = gpu_multipole(gpu_lib, s, cat, float(g["min_size"]), float(g["max_size"]))
    assert np.array_equal(small["ntri"], base["ntri"])
    err = max_rel_err(small, {k: g["ref_" + k] for k in MP_OUT})
    for k, v in err.items():
        assert v <= TOL, f"{k}: {v:.3e}"


@pytest.mark.parametrize("tensor", ["1", "0"])
def test_multipole_contraction_paths(gpu_lib, monkeypatch, tensor):
    """The tcgen05 contraction (3xTF32, TMEM accumulators) and the FP32 CUDA-core one both
    reproduce the reference."""
    from cases3 import spec3
    monkeypatch.setenv("TCGPU_MP_TENSOR", tensor)
    for name in ("ggg_flat_mp", "ggg_flat_mp_n20", "ggg_sphere_mp"):
        s = spec3(name)
        g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
        cat = {k[3:]: g[k] for k in g.files if k.startswith("c1_")}
        out = gpu_multipole(gpu_lib, s, cat, float(g["min_size"]), float(g["max_size"]))
        assert np.array_equal(out["ntri"], g["ref_ntri"]), name
        err = max_rel_err(out, {k: g["ref_" + k] for k in MP_OUT})
        for k, v in err.items():
            assert v <= TOL, f"{name} {k} tensor={tensor}: {v:.3e}"


@pytest.mark.parametrize("name", ["nnn_flat_mp", "nnn_sphere_mp"])
def test_multipole_nnn_golden(gpu_lib, name):
    """NNN LogMultipole through NNNCorr on an N field against the reference's NNNCorr."""
    from cases3 import spec3
    T = gpu_lib
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    s = spec3(str(g["case"]))
    cat = {k[3:]: g[k] for k in g.files if k.startswith("c1_")}
    nb, mn = s["nbins"], s["max_n"]
    shape = (nb, nb, 2 * mn + 1)
    keys = ("meand1", "meanlogd1", "meand2", "meanlogd2", "meand3", "meanlogd3", "meanu",
            "meanv", "weight", "weight_im", "ntri")
    out = {k: np.zeros(shape) for k in keys}
    e = np.array([])
    corr = T.NNNCorr(T.LogMultipole, s["min_sep"], s["max_sep"], nb, s["bin_size"], s["b"],
                     s["a"], 0., 0., mn, 0., 0., 0., 0., 0, 0., 0.,
                     -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
                     e, e, e, e, e, e, e, e, *[out[k] for k in keys])
    f = H.gpu_field(T, "N", s["coords"], cat, float(g["min_size"]), float(g["max_size"]))
    m = T.Euclidean if s["metric"] == "Euclidean" else T.Arc
    corr.processAuto(f, False, False, m)
    assert np.array_equal(out["ntri"], g["ref_ntri"]), name
    for k in ("weight", "weight_im", "meand2", "meanlogd2", "meand3", "meanlogd3"):
        r = g["ref_" + k]
        err = np.abs(out[k] - r).max() / max(np.abs(r).max(), 1e-300)
        assert err <= TOL, f"{name} {k}: {err:.3e}"
    # A G field is refused by NNN (and an N field by GGG).
    fg = H.gpu_field(T, "G", s["coords"], cat, float(g["min_size"]), float(g["max_size"]))
    with pytest.raises(ValueError):
        corr.processAuto(fg, False, False, m)


@pytest.mark.parametrize("name", ["kkk_flat_mp", "kkk_sphere_mp"])
def test_multipole_kkk_golden(gpu_lib, name):
    """KKK LogMultipole through KKKCorr on a K field against the reference's KKKCorr."""
    from cases3 import spec3
    T = gpu_lib
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    s = spec3(str(g["case"]))
    cat = {k[3:]: g[k] for k in g.files if k.startswith("c1_")}
    nb, mn = s["nbins"], s["max_n"]
    shape = (nb, nb, 2 * mn + 1)
    keys = ("zeta", "zeta_im", "meand1", "meanlogd1", "meand2", "meanlogd2", "meand3",
            "meanlogd3", "meanu", "meanv", "weight", "weight_im", "ntri")
    out = {k: np.zeros(shape) for k in keys}
    e = np.array([])
    corr = T.KKKCorr(T.LogMultipole, s["min_sep"], s["max_sep"], nb, s["bin_size"], s["b"],
                     s["a"], 0., 0., mn, 0., 0., 0., 0., 0, 0., 0.,
                     -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
                     out["zeta"], out["zeta_im"], e, e, e, e, e, e, *[out[k] for k in keys[2:]])
    f = H.gpu_field(T, "K", s["coords"], cat, float(g["min_size"]), float(g["max_size"]))
    m = T.Euclidean if s["metric"] == "Euclidean" else T.Arc
    corr.processAuto(f, False, False, m)
    assert np.array_equal(out["ntri"], g["ref_ntri"]), name
    for k in ("zeta", "zeta_im", "weight", "weight_im", "meand2", "meanlogd2", "meand3",
              "meanlogd3"):
        r = g["ref_" + k]
        err = np.abs(out[k] - r).max() / max(np.abs(r).max(), 1e-300)
        assert err <= TOL, f"{name} {k}: {err:.3e}"


def _corr3(T, letters, s):
    """A GGG / NNN / KKK LogMultipole object with its outputs (the reference's argument
    order, src/Corr3.cpp:4207-4225)."""
    nb, mn = s["nbins"], s["max_n"]
    shape = (nb, nb, 2 * mn + 1)
    common = ("meand1", "meanlogd1", "meand2", "meanlogd2", "meand3", "meanlogd3", "meanu",
              "meanv", "weight", "weight_im", "ntri")
    nG = letters.count("G")
    zk = (MP_OUT[:8] if nG == 3 else () if letters == "NNN" else MP_OUT[:4] if nG == 2
          else ("zeta", "zeta_im"))
    out = {k: np.zeros(shape) for k in zk + common}
    e = np.array([])
    zeta = [out[k] for k in zk] + [e] * (8 - len(zk))
    cls = getattr(T, letters + "Corr")
    corr = cls(T.LogMultipole, s["min_sep"], s["max_sep"], nb, s["bin_size"], s["b"], s["a"],
               0., 0., mn, 0., 0., 0., 0., 0, 0., 0., -sys.float_info.max, sys.float_info.max,
               0., 0., 0., *zeta, *[out[k] for k in common])
    return corr, out, zk


@pytest.mark.parametrize("name", ["ggg_flat_mp_x12", "ggg_sphere_mp_x12", "nnn_flat_mp_x12",
                                  "kkk_sphere_mp_x12", "nkk_flat_mp_x12", "knn_sphere_mp_x12",
                                  "ngg_flat_mp_x12", "ngg_sphere_mp_x12", "kgg_sphere_mp_x12",
                                  "gnn_flat_mp_x12", "gnn_sphere_mp_x12", "gkk_sphere_mp_x12"])
def test_multipole_cross12_golden(gpu_lib, name):
    """processCross12 (ordered = 1): vertex 1 from the first catalog, vertices 2 and 3 from
    the second, against the reference's own processCross12."""
    from cases3 import spec3
    T = gpu_lib
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    s = spec3(str(g["case"]))
    letters = str(g["letters"])
    cats = [{k[3:]: g[k] for k in g.files if k.startswith(p)} for p in ("c1_", "c2_")]
    f1, f2 = [H.gpu_field(T, L, s["coords"], c, float(g["min_size"]), float(g["max_size"]))
              for L, c in zip(letters[:2], cats)]
    m = T.Euclidean if s["metric"] == "Euclidean" else T.Arc
    corr, out, zk = _corr3(T, letters, s)
    corr.processCross12(f1, f2, 1, False, False, m)
    assert np.array_equal(out["ntri"], g["ref_ntri"]), name
    for k in zk + ("weight", "weight_im", "meand2", "meanlogd2", "meand3", "meanlogd3"):
        r = g["ref_" + k]
        err = np.abs(out[k] - r).max() / max(np.abs(r).max(), 1e-300)
        assert err <= TOL, f"{name} {k}: {err:.3e}"
    # Fields of another data kind are refused (vertex 1 and the pair field swapped, or a G
    # field in place of an N one), and so is processAuto for a mixed class.
    other = "N" if letters[1] != "N" else "G"
    fo = H.gpu_field(T, other, s["coords"], cats[1], float(g["min_size"]), float(g["max_size"]))
    with pytest.raises(ValueError):
        corr.processCross12(f1, fo, 1, False, False, m)
    if letters[0] != letters[1]:
        with pytest.raises(ValueError):
            corr.processCross12(f2, f1, 1, False, False, m)
        with pytest.raises(ValueError):
            corr.processAuto(f1, False, False, m)


def test_multipole_cross12_self_equals_auto(gpu_lib):
    """cross12 of a catalog with a second field built from the same catalog is its
    auto-correlation: the same triangles (ntri exact) and the same sums up to their order."""
    from cases3 import spec3
    T = gpu_lib
    name = "ggg_flat_mp"
    s = spec3(name)
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    cat = {k[3:]: g[k] for k in g.files if k.startswith("c1_")}
    f1 = H.gpu_field(T, "G", s["coords"], cat, float(g["min_size"]), float(g["max_size"]))
    f2 = H.gpu_field(T, "G", s["coords"], cat, float(g["min_size"]), float(g["max_size"]))
    corr, out, _ = _corr3(T, "GGG", s)
    corr.processCross12(f1, f2, 1, False, False, T.Euclidean)
    assert np.array_equal(out["ntri"], g["ref_ntri"])
    err = max_rel_err(out, {k: g["ref_" + k] for k in MP_OUT})
    for k, v in err.items():
        assert v <= TOL, f"{k}: {v:.3e}"


@pytest.mark.parametrize("name", ["ngg_flat_mp_x12", "kgg_sphere_mp_x12", "gkk_sphere_mp_x12"])
def test_multipole_cross12_cuda_core_contraction(gpu_lib, monkeypatch, name):
    """NGG / KGG (G_n at n, no +-1 buffer) and GKK (real pair payload) through the FP32
    CUDA-core contraction as well as the tensor-core one."""
    from cases3 import spec3
    T = gpu_lib
    monkeypatch.setenv("TCGPU_MP_TENSOR", "0")
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    s = spec3(str(g["case"]))
    letters = str(g["letters"])
    cats = [{k[3:]: g[k] for k in g.files if k.startswith(p)} for p in ("c1_", "c2_")]
    f1, f2 = [H.gpu_field(T, L, s["coords"], c, float(g["min_size"]), float(g["max_size"]))
              for L, c in zip(letters[:2], cats)]
    m = T.Euclidean if s["metric"] == "Euclidean" else T.Arc
    corr, out, zk = _corr3(T, letters, s)
    corr.processCross12(f1, f2, 1, False, False, m)
    assert np.array_equal(out["ntri"], g["ref_ntri"]), name
    for k in zk + ("weight", "weight_im"):
        r = g["ref_" + k]
        err = np.abs(out[k] - r).max() / max(np.abs(r).max(), 1e-300)
        assert err <= TOL, f"{name} {k}: {err:.3e}"


def _x3_run(T, g, s):
    """The fixture's processCross / processCross21 / processCross12(ordered = 0) call on the
    GPU module."""
    letters, call, ordered = str(g["letters"]), str(g["call"]), int(g["ordered"])
    kinds = {"cross": letters, "cross21": letters[0] + letters[2], "cross12": letters[:2]}[call]
    cats = [{k[3:]: g[k] for k in g.files if k.startswith(f"c{i + 1}_")} for i in range(len(kinds))]
    fs = [H.gpu_field(T, L, s["coords"], c, float(g["min_size"]), float(g["max_size"]))
          for L, c in zip(kinds, cats)]
    m = T.Euclidean if s["metric"] == "Euclidean" else T.Arc
    corr, out, zk = _corr3(T, letters, s)
    if call == "cross":
        corr.processCross(fs[0], fs[1], fs[2], ordered, False, False, m)
    elif call == "cross21":
        corr.processCross21(fs[0], fs[1], ordered, False, False, m)
    else:
        corr.processCross12(fs[0], fs[1], ordered, False, False, m)
    return out, zk


@pytest.mark.parametrize("name", ["ggg_flat_mp_x3o4", "ggg_sphere_mp_x3o1", "ggg_flat_mp_x21o3",
                                  "kkk_flat_mp_x3o0", "nnn_sphere_mp_x12o0", "ngg_flat_mp_x3o4",
                                  "gkk_sphere_mp_x3o1", "nnk_flat_mp_x21o3", "nkn_sphere_mp_x3o4",
                                  "knk_flat_mp_x3o4", "kkn_sphere_mp_x21o3", "nng_flat_mp_x21o3",
                                  "ngn_sphere_mp_x3o4", "kkg_sphere_mp_x21o3", "kgk_flat_mp_x3o4",
                                  "gng_flat_mp_x3o4", "ggn_sphere_mp_x21o3", "gkg_sphere_mp_x3o4",
                                  "ggk_flat_mp_x21o3", "ggg_flat_mp_x3o2", "nnn_flat_mp_x3o3",
                                  "kkk_sphere_mp_x21o0"])
@pytest.mark.parametrize("tensor", ["1", "0"])
def test_multipole_three_field_golden(gpu_lib, monkeypatch, name, tensor):
    """The three-field multipole (vertex 2's pairs in bins [0, nb), vertex 3's in [nb, 2 nb)
    of one scratch) through processCross / processCross21 / processCross12(ordered = 0),
    against the reference's own calls, on the tensor-core and the CUDA-core contraction."""
    from cases3 import spec3
    monkeypatch.setenv("TCGPU_MP_TENSOR", tensor)
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    s = spec3(str(g["case"]))
    out, zk = _x3_run(gpu_lib, g, s)
    assert np.array_equal(out["ntri"], g["ref_ntri"]), name
    for k in zk + ("weight", "weight_im", "meand2", "meanlogd2", "meand3", "meanlogd3"):
        r = g["ref_" + k]
        err = np.abs(out[k] - r).max() / max(np.abs(r).max(), 1e-300)
        assert err <= TOL, f"{name} {k}: {err:.3e}"


def test_multipole_three_field_inplace(gpu_lib, monkeypatch):
    """A record buffer of a few vertices sends most vertex records of a three-field cross to
    the in-place FP64 contraction; the result must not change."""
    from cases3 import spec3
    monkeypatch.setenv("TCGPU_MP_RECORD_BYTES", str(40 * 16 * 1024))
    name = "ggg_sphere_mp_x3o1"
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    s = spec3(str(g["case"]))
    out, zk = _x3_run(gpu_lib, g, s)
    assert np.array_equal(out["ntri"], g["ref_ntri"])
    for k in zk + ("weight", "weight_im", "meand2", "meanlogd2", "meand3", "meanlogd3"):
        r = g["ref_" + k]
        err = np.abs(out[k] - r).max() / max(np.abs(r).max(), 1e-300)
        assert err <= TOL, f"{k}: {err:.3e}"


def test_multipole_three_field_many_bins(gpu_lib):
    """NNG through processCross21 (ordered 3) with 20 bins (40 scratch bins: the CUDA-core
    contraction and the larger shared-memory tiles) against the oracle on the same points."""
    from oracle import oracle as O
    T = gpu_lib
    rng = np.random.default_rng(515)
    n, side = 1500, 60.0
    cn = {"x": rng.uniform(0, side, n), "y": rng.uniform(0, side, n), "w": rng.uniform(0.5, 1.5, n)}
    cg = {"x": rng.uniform(0, side, n), "y": rng.uniform(0, side, n), "w": rng.uniform(0.5, 1.5, n),
          "g1": rng.normal(0, 0.2, n), "g2": rng.normal(0, 0.2, n)}
    lo, hi, nb, mn = 1.0, 20.0, 20, 8
    bs = np.log(hi / lo) / nb
    s = dict(coords="flat", metric="Euclidean", min_sep=lo, max_sep=hi, nbins=nb, max_n=mn,
             bin_size=bs, b=min(bs, 0.1), a=np.pi / (2 * mn + 1))
    b1 = min(s["a"], s["b"])
    mins, maxs = 2 * lo * b1 / (2 + 3 * b1), hi * b1
    corr, out, zk = _corr3(T, "NNG", s)
    fN = H.gpu_field(T, "N", "flat", dict(cn, z=None), mins, maxs)
    fG = H.gpu_field(T, "G", "flat", dict(cg, z=None), mins, maxs)
    corr.processCross21(fN, fG, 3, False, False, T.Euclidean)
    args = (mins, maxs, "mean", False, 3, 10)
    on = O.OracleField("K", "flat", cn["x"], cn["y"], None, np.ones(n), None, cn["w"], None, *args)
    og = O.OracleField("G", "flat", cg["x"], cg["y"], None, cg["g1"], cg["g2"], cg["w"], None,
                       *args)
    bins = dict(min_sep=lo, max_sep=hi, nbins=nb, bin_size=bs, b=s["b"], a=s["a"])
    ref = O.multipole3("Euclidean", bins, mn, on, on, og, 4, nthreads=0, mode=3)
    assert np.array_equal(out["ntri"], ref["ntri"])
    assert out["ntri"].sum() > 0
    for mine, r in (("zeta", "gam0r"), ("zeta_im", "gam0i"), ("weight", "weight"),
                    ("meand2", "meand2"), ("meanlogd3", "meanlogd3")):
        err = np.abs(out[mine] - ref[r]).max() / max(np.abs(ref[r]).max(), 1e-300)
        assert err <= TOL, f"{mine}: {err:.3e}"


def test_multipole_three_field_edge_cases(gpu_lib):
    """An empty field leaves the outputs untouched (the reference's loops do nothing); an
    ordered value the reference's dispatch has no case for, or fields in different coordinate
    systems, are refused."""
    from cases3 import spec3
    T = gpu_lib
    name = "ggg_flat_mp_x3o4"
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz"))
    s = spec3(str(g["case"]))
    cats = [{k[3:]: g[k] for k in g.files if k.startswith(f"c{i + 1}_")} for i in range(3)]
    fs = [H.gpu_field(T, "G", "flat", c, float(g["min_size"]), float(g["max_size"])) for c in cats]
    empty = {k: v[:0] for k, v in cats[2].items()}
    fe = H.gpu_field(T, "G", "flat", empty, float(g["min_size"]), float(g["max_size"]))
    corr, out, zk = _corr3(T, "GGG", s)
    corr.processCross(fs[0], fs[1], fe, 4, False, False, T.Euclidean)
    corr.processCross21(fe, fs[1], 3, False, False, T.Euclidean)
    corr.processCross12(fs[0], fe, 0, False, False, T.Euclidean)
    for k, v in out.items():
        assert not np.any(v), k
    with pytest.raises(ValueError):
        corr.processCross21(fs[0], fs[1], 1, False, False, T.Euclidean)
    with pytest.raises(ValueError):
        corr.processCross(fs[0], fs[1], fs[2], 5, False, False, T.Euclidean)
    with pytest.raises(ValueError):
        corr.processCross12(fs[0], fs[1], 2, False, False, T.Euclidean)
    sph = {"x": cats[2]["x"] * 0 + 1.0, "y": cats[2]["y"] * 0, "z": cats[2]["x"] * 0,
           "g1": cats[2]["g1"], "g2": cats[2]["g2"], "w": cats[2]["w"]}
    fsph = H.gpu_field(T, "G", "spherical", sph, 0.0, 0.0)
    with pytest.raises(ValueError):
        corr.processCross(fs[0], fs[1], fsph, 4, False, False, T.Euclidean)
