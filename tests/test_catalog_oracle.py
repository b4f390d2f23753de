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


def test_wrapper_rejects_bad_columns():
    """The module's catalog_finish checks its columns before any device work: unknown names
    and columns of different lengths are ValueErrors."""
    from treecorr_gb300 import _treecorr as T
    x = np.arange(5.)
    with pytest.raises(ValueError, match="unknown column"):
        T.catalog_finish({"x": x, "y": x, "colour": x})
    with pytest.raises(ValueError, match="lengths"):
        T.catalog_finish({"x": x, "y": x[:4]})
    with pytest.raises(ValueError, match="length"):
        T.catalog_finish({"x": x, "y": x}, w=np.ones(4))


def test_oracle_flag_and_nan_order():
    """The reference's order of the steps: a NaN in w on a row that a NaN in x already zeroed
    is not counted for w; a flagged row's NaN weight is not counted either."""
    from oracle import catalog_oracle as O
    x = np.array([0., np.nan, 2., 3.])
    w = np.array([1., np.nan, np.nan, 1.])
    flag = np.array([0, 0, 4, 0])
    cols, gw, _, info = O.finish_input({"x": x, "y": np.zeros(4)}, w=w, flag=flag,
                                       keep_zero_weight=True)
    assert info["nan_counts"]["x"] == 1 and info["nan_counts"]["w"] == 0
    np.testing.assert_array_equal(gw, [1., 0., 0., 1.])
    assert info["sumw"] == 2.0 and info["nobj"] == 2
