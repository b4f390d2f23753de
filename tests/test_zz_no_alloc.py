"""GPU test of tc_corr2_process_auto_noalloc, the allocation-free auto-correlation.

Some callers cannot let this library allocate GPU memory while it runs: a process whose
device memory is all handed out by its own memory pool, or a latency-critical pipeline that
must not take the device-wide synchronisation cudaMalloc/cudaFree can cause.  For them the
library offers one entry point that allocates nothing: it uses a fixed device array that is
part of the library.  This test calls it through the C ABI, twice in a row, and checks each result
against tc_corr2_process_auto on the same field, and that free device memory does not
change across the calls.

The file name makes pytest collect it last.
"""
import ctypes

import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu


def _noalloc_fn(T):
    L = T.lib()
    fn = L.tc_corr2_process_auto_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    return L, fn


def _corr(T, dtype, bins, out):
    import sys
    e = np.array([])
    xi = [out["xi0"], out["xi1"], out["xi2"], out["xi3"]]
    if dtype == "N":
        xi = [e, e, e, e]
    elif dtype == "K":
        xi = [out["xi0"], e, e, e]
    return getattr(T, dtype * 2 + "Corr")(T.Log, bins["min_sep"], bins["max_sep"],
                                          bins["nbins"], bins["bin_size"], bins["b"], bins["a"],
                                          -sys.float_info.max, sys.float_info.max, 0., 0., 0.,
                                          *xi, out["meanr"], out["meanlogr"], out["weight"],
                                          out["npairs"])


@pytest.mark.parametrize("name", ["gg_flat_bs1", "gg_sphere_arc", "nn_flat_bs1", "kk_flat_bs0"])
def test_noalloc_matches_process_auto(gpu_lib, name):
    import torch
    T = gpu_lib
    L, noalloc = _noalloc_fn(T)
    s, c1, c2, bins, min_size, max_size, golden = H.load_case(name)
    f = H.gpu_field(T, s["dtype"], s["coords"], c1, min_size, max_size, s["split"], s["brute"],
                    s["min_top"], s["max_top"])
    f.getNTopLevel()    # build the tree first: building allocates
    ref = H.gpu_process(T, s["dtype"], s["metric"], bins, f)
    metric = int(T.Euclidean if s["metric"] == "Euclidean" else T.Arc)
    outs = [{k: np.zeros(bins["nbins"]) for k in H.OUT_KEYS} for _ in range(2)]
    corrs = [_corr(T, s["dtype"], bins, o) for o in outs]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for corr in corrs:
        rc = noalloc(corr._h, f._h, 0, metric)
        assert rc == 0, L.tc_last_error().decode()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, f"device memory changed by {free0 - free1} bytes"
    for out in outs:
        # Same kernels and decisions; only the grouping of FP32 partials into warps differs.
        H.assert_outputs_close(out, ref, s["dtype"], rtol=1e-6, label=name + " noalloc")
        H.assert_outputs_close(out, golden, s["dtype"], rtol=1e-5, label=name + " golden")


def test_noalloc_rejects_what_it_cannot_hold(gpu_lib):
    T = gpu_lib
    L, noalloc = _noalloc_fn(T)
    s, c1, c2, bins, min_size, max_size, golden = H.load_case("nn_flat_bs1")
    # A field whose tree is not built yet (building would allocate).
    f = H.gpu_field(T, "N", "flat", c1, min_size, max_size)
    out = {k: np.zeros(bins["nbins"]) for k in H.OUT_KEYS}
    corr = _corr(T, "N", bins, out)    # keep the object alive while its handle is used
    rc = noalloc(corr._h, f._h, 0, int(T.Euclidean))
    assert rc == 1 and b"not built" in L.tc_last_error()
    # More bins than the fixed scratch holds.
    f.getNTopLevel()
    big = dict(bins, nbins=100, bin_size=np.log(bins["max_sep"] / bins["min_sep"]) / 100)
    out = {k: np.zeros(100) for k in H.OUT_KEYS}
    corr_big = _corr(T, "N", big, out)
    rc = noalloc(corr_big._h, f._h, 0, int(T.Euclidean))
    assert rc == 1 and b"at most 64" in L.tc_last_error()
    assert not out["npairs"].any()


def test_noalloc_refuses_the_learned_criterion(gpu_lib):
    """The allocation-free call runs the bin_slop criterion only: a corr that has the learned
    criterion set is refused with a clear message and its outputs stay untouched."""
    T = gpu_lib
    L, noalloc = _noalloc_fn(T)
    s, c1, c2, bins, min_size, max_size, golden = H.load_case("gg_flat_bs1")
    f = H.gpu_field(T, "G", "flat", c1, min_size, max_size)
    f.getNTopLevel()
    out = {k: np.zeros(bins["nbins"]) for k in H.OUT_KEYS}
    corr = _corr(T, "G", bins, out)
    corr.setLearned(np.zeros(T.mlp_nparam(), dtype=np.float32), threshold=-3.0)
    rc = noalloc(corr._h, f._h, 0, int(T.Euclidean))
    assert rc == 1 and b"bin_slop criterion only" in L.tc_last_error()
    assert not out["weight"].any() and not out["npairs"].any()
    corr.setLearned(None)   # back to the plain criterion: accepted again
    rc = noalloc(corr._h, f._h, 0, int(T.Euclidean))
    assert rc == 0, L.tc_last_error().decode()
    H.assert_outputs_close(out, golden, "G", rtol=1e-5, label="after setLearned(None)")


def test_noalloc_work_list_overflow_is_reported(gpu_lib, monkeypatch):
    """When the traversal needs more spill-list space than the fixed array holds, the kernel
    stops with a status (no write past the list), the call returns TC_ERR_DEVICE with the
    documented message and adds nothing to the outputs.  The test shortens the list
    (TCGPU_NOALLOC_SPILL_CAP) so that a 200,000-point catalog reaches that path."""
    from cases_bench import bench2_inputs, bench2_spec
    T = gpu_lib
    L, noalloc = _noalloc_fn(T)
    s = bench2_spec("gg_cfg1_bs1")
    f = H.gpu_field(T, "G", s["coords"], bench2_inputs("gg_cfg1_bs1"), s["min_size"],
                    s["max_size"])
    f.getNTopLevel()
    out = {k: np.zeros(s["bins"]["nbins"]) for k in H.OUT_KEYS}
    c = _corr(T, "G", s["bins"], out)
    monkeypatch.setenv("TCGPU_NOALLOC_SPILL_CAP", "0")
    rc = noalloc(c._h, f._h, 0, int(T.Euclidean))
    assert rc == 4    # TC_ERR_DEVICE
    assert "work-list space" in L.tc_last_error().decode()
    assert not any(out[k].any() for k in H.OUT_KEYS)
    # The same call with the full list succeeds and matches the golden result.
    monkeypatch.delenv("TCGPU_NOALLOC_SPILL_CAP")
    assert noalloc(c._h, f._h, 0, int(T.Euclidean)) == 0
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                             "gg_cfg1_bs1.npz"))
    H.assert_outputs_close(out, {k: g["ref_" + k] for k in H.OUT_KEYS}, "G", rtol=1e-5,
                           label="noalloc after an overflow")
