"""Bitwise repeatability of the 2-point path (the reference's results repeat exactly at
num_threads=1, tests/test_gg.py:573-574).

With the fixed-order expansion (the default) the children and tiles of every expansion
launch are joined in warp order, so each warp takes the same items in every run and every
floating-point sum is formed in the same order: repeated calls agree bit for bit, on the
bin_slop traversal, the exact-mode tiles and the learned criterion alike.  With it off the
results still equal the reference's (the golden outputs) and agree with the fixed-order ones
to rounding."""
import os

import numpy as np
import pytest

import helpers as H
from cases_bench import bench2_inputs, bench2_spec

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _bench_case(T, name):
    s = bench2_spec(name)
    cat = bench2_inputs(name)
    f = H.gpu_field(T, "G", s["coords"], cat, s["min_size"], s["max_size"])
    g = np.load(os.path.join(HERE, name + ".npz"))
    return s, f, {k: g["ref_" + k] for k in H.OUT_KEYS}


@pytest.fixture
def det_switch(gpu_lib):
    prev = gpu_lib.SetDeterministic(True)
    yield gpu_lib
    gpu_lib.SetDeterministic(prev)


@pytest.mark.parametrize("name", ["gg_cfg2_bs01", "gg_cfg2_exact", "gg_cfg1_bs1"])
def test_repeats_bit_identical(det_switch, name):
    """Three runs on the 200K-point benchmark-shape catalogs (several expansion launches;
    the exact case through the leaf-pair tiles): every output array identical, and equal to
    the reference's within the parity bound."""
    T = det_switch
    s, f, ref = _bench_case(T, name)
    runs = [H.gpu_process(T, "G", s["metric"], s["bins"], f) for _ in range(3)]
    assert runs[0]["_stats"]["launches"] > 1
    for r in runs[1:]:
        for k in H.OUT_KEYS:
            assert np.array_equal(r[k], runs[0][k]), (name, k)
    H.assert_outputs_close(runs[0], ref, "G", rtol=1e-5, label=name)


def test_fixed_order_off_still_parity(det_switch):
    """Arrival order (the switch off): the reference's outputs within the parity bound, and
    the fixed-order result within FP32 rounding of it."""
    T = det_switch
    s, f, ref = _bench_case(T, "gg_cfg2_bs01")
    a = H.gpu_process(T, "G", s["metric"], s["bins"], f)
    assert T.SetDeterministic(False) is True
    assert not T.GetDeterministic()
    b = H.gpu_process(T, "G", s["metric"], s["bins"], f)
    H.assert_outputs_close(b, ref, "G", rtol=1e-5, label="arrival order")
    assert np.array_equal(a["npairs"], b["npairs"])
    # The two orders group the FP32 partials differently: agreement to FP32 rounding of the
    # array's scale (the parity bound is 1e-5).
    for k in ("weight", "xi0", "xi2", "meanr", "meanlogr"):
        np.testing.assert_allclose(a[k], b[k], rtol=0, atol=1e-6 * np.abs(a[k]).max())


def test_learned_repeats_bit_identical(det_switch):
    """The learned criterion (network inference inside the traversal) repeats bit for bit."""
    T = det_switch
    from test_gpu_learned import _flat_setup, _run
    from treecorr_gb300 import learned as L
    cat, f, bins = _flat_setup(T)
    bins = dict(bins, b=0.1 * bins["bin_size"])
    params = L.init_params(seed=3)     # output bias -3: every candidate is accepted at 0
    a = _run(T, f, bins, params, threshold=0.0)
    b = _run(T, f, bins, params, threshold=0.0)
    assert a["_stats"]["learned"] > 0
    for k in H.OUT_KEYS:
        assert np.array_equal(a[k], b[k]), k


def test_pooled_level_buffers_reused_and_trimmed(det_switch):
    """Level buffers come from the stream-ordered pool: a second corr after the first is
    freed gives the same result, and TrimMemory returns the pool's memory."""
    import torch
    T = det_switch
    s, f, ref = _bench_case(T, "gg_cfg2_bs01")
    a = H.gpu_process(T, "G", s["metric"], s["bins"], f)
    b = H.gpu_process(T, "G", s["metric"], s["bins"], f)
    for k in H.OUT_KEYS:
        assert np.array_equal(a[k], b[k]), k
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    T.TrimMemory()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 >= free0
