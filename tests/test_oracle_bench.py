"""CPU tests: the oracle against the reference's outputs at the benchmark configurations'
own shapes and binnings (tests/golden/cases_bench.py), and the portable catalogs against the
input hashes stored with those outputs."""
import os

import numpy as np
import pytest

import helpers as H
from cases_bench import (BENCH2, BENCH3, bench2_inputs, bench2_spec, bench3_inputs,
                         bench3_spec, catalog_hash)

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", sorted(BENCH2) + sorted(BENCH3))
def test_portable_catalog_hash(name):
    g = np.load(os.path.join(HERE, name + ".npz"))
    cat = bench2_inputs(name) if name in BENCH2 else bench3_inputs(name)
    assert catalog_hash(cat) == str(g["input_sha256"])


@pytest.mark.parametrize("name", sorted(BENCH2))
def test_oracle_matches_reference_bench(name):
    s = bench2_spec(name)
    g = np.load(os.path.join(HERE, name + ".npz"))
    cat = bench2_inputs(name)
    f = H.oracle_field("G", s["coords"], cat, s["min_size"], s["max_size"], s["split"],
                       s["brute"], s["min_top"], s["max_top"])
    assert f.ntop() == int(g["ntop"])
    # Every host core (an earlier import of torch may have lowered OpenMP's default).
    out = H.oracle_process("G", s["metric"], s["bins"], f, nthreads=os.cpu_count() or 1)
    assert np.array_equal(out["npairs"], g["ref_npairs"])
    for k in H.OUT_KEYS:
        r = g["ref_" + k]
        scale = max(np.abs(r).max(), 1e-300)
        # All host threads here, one in the reference run: the summation order differs.
        assert np.abs(out[k] - r).max() <= 1e-10 * scale, k


def test_oracle_multipole_matches_reference_cfg4():
    from oracle import oracle as O
    name = "ggg_cfg4"
    s = bench3_spec(name)
    g = np.load(os.path.join(HERE, name + ".npz"))
    cat = bench3_inputs(name)
    f = H.oracle_field("G", "flat", cat, s["min_size"], s["max_size"])
    bins = {k: s[k] for k in ("min_sep", "max_sep", "nbins", "bin_size", "b", "a")}
    out = O.multipole(s["metric"], bins, s["max_n"], f, nthreads=os.cpu_count() or 1)
    assert np.array_equal(out["ntri"], g["ref_ntri"])
    for k in O.MP_KEYS:
        r = g["ref_" + k]
        scale = max(np.abs(r).max(), 1e-300)
        assert np.abs(out[k] - r).max() <= 1e-10 * scale, k
