"""GPU parity at the benchmark configurations' own shapes and binnings, against outputs of
the reference C++ (tests/golden/cases_bench.py):

  * flat GG on 200,000 points with 20 Log bins 1-100' at bin_slop 1, 0 and 0 / angle_slop 0
    (the reference's tests/test_gg.py:25-128 pins the same quantities on smaller catalogs);
  * curved-sky GG on a 200,000-point sample of the 1000 deg^2 cap, Arc, 30 Log bins 1-300',
    at bin_slop 0.1, 0 and 0 / angle_slop 0;
  * GGG LogMultipole with 20 bins 1-50' and max_n 30 on both contraction paths (the tcgen05
    one then has 4 x 20 = 80 live columns; tests/test_ggg.py:4441-4558 pins the multipole).

The catalogs are regenerated bit-identically from their seeds; each test first checks the
SHA-256 of the inputs against the one stored with the reference's outputs.
"""
import os
import sys

import numpy as np
import pytest

import helpers as H
from cases_bench import (BENCH2, bench2_inputs, bench2_spec, bench3_inputs, bench3_spec,
                         catalog_hash)

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

RTOL = 1e-5   # xi, weight, meanr, meanlogr: max |gpu - ref| / scale; npairs bit-identical


def _golden(name):
    return np.load(os.path.join(HERE, name + ".npz"))


@pytest.mark.parametrize("name", sorted(BENCH2))
@pytest.mark.parametrize("tiles", ["1", "0"])
def test_bench2_golden(gpu_lib, monkeypatch, name, tiles):
    """bin_slop > 0 runs the plain traversal (tiles does not apply); the exact cases run the
    leaf-pair tiles (tiles=1) and the traversal down to the leaves (tiles=0)."""
    s = bench2_spec(name)
    exact = s["bins"]["a"] == 0.
    if tiles == "0" and not exact:
        pytest.skip("the tile switch only matters in exact mode")
    monkeypatch.setenv("TCGPU_TILES", tiles)
    T = gpu_lib
    g = _golden(name)
    cat = bench2_inputs(name)
    assert catalog_hash(cat) == str(g["input_sha256"]), "regenerated catalog differs"
    f = H.gpu_field(T, "G", s["coords"], cat, s["min_size"], s["max_size"], s["split"],
                    s["brute"], s["min_top"], s["max_top"])
    assert f.getNTopLevel() == int(g["ntop"])
    got = H.gpu_process(T, "G", s["metric"], s["bins"], f)
    ref = {k: g["ref_" + k] for k in H.OUT_KEYS}
    H.assert_outputs_close(got, ref, "G", rtol=RTOL, label=f"{name} tiles={tiles}")
    st = got["_stats"]
    if exact and tiles == "1":
        assert st["tiles"] > 0 and st["tile_pairs"] > 0
        # Every accepted pair of the exact mode is a leaf pair at its own separation.
        assert st["accepted"] == int(ref["npairs"].sum())
    else:
        assert st["tiles"] == 0
    print(name, tiles, {k: st[k] for k in ("cell_pairs", "accepted", "tiles", "tile_pairs",
                                           "tile_escalated", "traverse_ms")})


@pytest.mark.parametrize("tensor", ["1", "0"])
def test_ggg_cfg4_golden(gpu_lib, monkeypatch, tensor):
    """nbins 20, max_n 30: NC = 80 columns in the tensor-core contraction (tensor=1) and the
    FP32 CUDA-core contraction (tensor=0)."""
    from test_gpu_multipole import MP_OUT, TOL, gpu_multipole, max_rel_err
    monkeypatch.setenv("TCGPU_MP_TENSOR", tensor)
    name = "ggg_cfg4"
    s = bench3_spec(name)
    g = _golden(name)
    cat = bench3_inputs(name)
    assert catalog_hash(cat) == str(g["input_sha256"]), "regenerated catalog differs"
    out = gpu_multipole(gpu_lib, s, cat, s["min_size"], s["max_size"])
    assert np.array_equal(out["ntri"], g["ref_ntri"])
    err = max_rel_err(out, {k: g["ref_" + k] for k in MP_OUT})
    print(name, tensor, " ".join(f"{k}={v:.1e}" for k, v in err.items() if v > 0))
    for k, v in err.items():
        assert v <= TOL, f"{name} tensor={tensor} {k}: {v:.3e}"
