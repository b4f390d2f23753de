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


@pytest.mark.parametrize("name", CC.NAMES)
def test_center_size_matches_reference(name):
    """Catalog._get_center_size of the finished catalog: the oracle's restatement equals the
    reference's values."""
    from oracle import catalog_oracle as O
    _, _, out, ref = CC.load(name)
    got = O.center_size(out["x"], out["y"], out.get("z"))
    np.testing.assert_allclose(got, ref["center_size"], rtol=0,
                               atol=1e-14 * max(1.0, np.abs(ref["center_size"]).max()))
