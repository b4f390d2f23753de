"""CPU: the oracle's restatement of Catalog._finish_input (oracle/catalog_oracle.py) against
TreeCorr's own Catalog on the fixtures (tests/golden/catalog_*.npz)."""
import numpy as np
import pytest

import catalog_cases as CC


def test_fixtures_present():
    assert len(CC.NAMES) >= 6


@pytest.mark.parametrize("name", CC.NAMES)
def test_oracle_matches_reference_catalog(name):
    from oracle import catalog_oracle as O
    cfg, inp, out, ref = CC.load(name)
    cols, w, wpos, flag = CC.split_inputs(inp)
    got, gw, gwpos, info = O.finish_input(cols, w, wpos, flag, **CC.flag_args(cfg))
    assert info["nontrivial_w"] == ref["nontrivial_w"]
    assert info["nobj"] == ref["nobj"]
    assert len(gw) == ref["ntot"]
    np.testing.assert_allclose(info["sumw"], ref["sumw"], rtol=1e-13)
    np.testing.assert_array_equal(gw, out["w"])
    if gwpos is not None:
        np.testing.assert_array_equal(gwpos, out["wpos"])
    for k, v in got.items():
        np.testing.assert_array_equal(v, out[k], err_msg=k)
    # The fixture really exercises the rules it is named for.
    if "nan" in name or name == "sky_radec":
        assert sum(info["nan_counts"].values()) > 0
    if name == "flat_wpos":
        assert info["wpos_zero"] > 0 and info["wpos_conflicts"] > 0
