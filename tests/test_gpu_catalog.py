"""GPU catalog ingestion (tc_catalog_finish / tc_catalog_finish_device) against TreeCorr's
own Catalog (tests/golden/catalog_*.npz) and the oracle: the flag -> weight conversion, the
NaN checks, the wpos == 0 rule, sumw and the removal of zero-weight rows
(treecorr/catalog.py:1343-1487); then GenerateXYZ on the cleaned sky columns."""
import numpy as np
import pytest

import catalog_cases as CC

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", CC.NAMES)
def test_host_columns_match_reference(gpu_lib, name):
    T = gpu_lib
    from oracle import catalog_oracle as O
    cfg, inp, out, ref = CC.load(name)
    cols, w, wpos, flag = CC.split_inputs(inp)
    got, gw, gwpos, info = T.catalog_finish(cols, w, wpos, flag, **CC.flag_args(cfg))
    assert info["nontrivial_w"] == ref["nontrivial_w"]
    assert info["nkeep"] == ref["ntot"] and info["nobj"] == ref["nobj"]
    np.testing.assert_allclose(info["sumw"], ref["sumw"], rtol=1e-13)
    np.testing.assert_array_equal(gw, out["w"])
    if gwpos is not None:
        np.testing.assert_array_equal(gwpos, out["wpos"])
    for k, v in got.items():
        np.testing.assert_array_equal(v, out[k], err_msg=k)
    _, _, _, oinfo = O.finish_input(cols, w, wpos, flag, **CC.flag_args(cfg))
    for k, c in oinfo["nan_counts"].items():
        assert info["nan_counts"][k] == c, k
    assert info["wpos_zero"] == oinfo["wpos_zero"]
    assert info["wpos_conflicts"] == oinfo["wpos_conflicts"]
    if "ra" in got:
        # Positions from the cleaned sky columns, as the reference's _generate_xyz.
        x, y, z = (np.empty(info["nkeep"]) for _ in range(3))
        T.GenerateXYZ(x, y, z, got["ra"], got["dec"], got.get("r", np.array([])))
        for k, v in (("x", x), ("y", y), ("z", z)):
            np.testing.assert_allclose(v, out[k], rtol=0, atol=4e-16 * np.abs(out[k]).max())


def test_device_columns_in_place(gpu_lib):
    """The device entry point on torch-held columns: compacted in place, same as the host
    one; repeated calls give the same sumw bit for bit."""
    import torch
    T = gpu_lib
    cfg, inp, out, ref = CC.load("flat_flags_nan")
    cols, w, wpos, flag = CC.split_inputs(inp)
    names = [k for k in T.CAT_COLUMNS if k in cols]
    sums = []
    for _ in range(2):
        d = {k: torch.from_numpy(np.array(cols[k])).cuda() for k in names}
        dw = torch.from_numpy(np.array(w)).cuda()
        dflag = torch.from_numpy(np.array(flag, dtype=np.int64)).cuda()
        info = T.catalog_finish_device(len(dw), [d[k].data_ptr() for k in names], dw.data_ptr(),
                                       flag_ptr=dflag.data_ptr(), names=names,
                                       **CC.flag_args(cfg))
        m = info["nkeep"]
        assert m == ref["ntot"]
        np.testing.assert_array_equal(dw[:m].cpu().numpy(), out["w"])
        for k in names:
            np.testing.assert_array_equal(d[k][:m].cpu().numpy(), out[k], err_msg=k)
        sums.append(info["sumw"])
    assert sums[0] == sums[1]


def test_zero_sumw_is_an_error(gpu_lib):
    T = gpu_lib
    x = np.arange(10.)
    with pytest.raises(ValueError, match="sumw == 0"):
        T.catalog_finish({"x": x, "y": x}, w=np.zeros(10))


def test_large_random_vs_oracle(gpu_lib):
    """2M rows (many blocks) with every rule active: equal to the oracle."""
    T = gpu_lib
    from oracle import catalog_oracle as O
    rng = np.random.default_rng(9)
    n = 2_000_000
    cols = {"x": rng.uniform(0, 1, n), "y": rng.uniform(0, 1, n), "k": rng.normal(0, 1, n)}
    for k in cols:
        cols[k][rng.choice(n, 500, replace=False)] = np.nan
    w = rng.uniform(0.5, 1.5, n)
    w[rng.choice(n, 1000, replace=False)] = 0.
    wpos = rng.uniform(0.5, 1.5, n)
    wpos[rng.choice(n, 700, replace=False)] = 0.
    flag = rng.integers(0, 16, n)
    a = T.catalog_finish(cols, w, wpos, flag, ok_flag=3)
    b = O.finish_input(cols, w, wpos, flag, ok_flag=3)
    for k in cols:
        np.testing.assert_array_equal(a[0][k], b[0][k], err_msg=k)
    np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(a[2], b[2])
    np.testing.assert_allclose(a[3]["sumw"], b[3]["sumw"], rtol=1e-12)
    assert a[3]["nobj"] == b[3]["nobj"] and a[3]["nkeep"] == len(b[1])


@pytest.mark.parametrize("name", CC.NAMES)
def test_center_size_matches_reference(gpu_lib, name):
    """The finished catalog's centre and size (what triviallyZero compares) on the GPU, host
    and device entry points, against the reference's _get_center_size."""
    import torch
    T = gpu_lib
    _, _, out, ref = CC.load(name)
    z = out.get("z")
    got = T.catalog_center_size(out["x"], out["y"], z)
    tol = 1e-13 * max(1.0, np.abs(ref["center_size"]).max())
    np.testing.assert_allclose(got, ref["center_size"], rtol=0, atol=tol)
    d = [torch.from_numpy(np.array(a)).cuda() for a in (out["x"], out["y"])]
    dz = torch.from_numpy(np.array(z)).cuda() if z is not None else None
    got2 = T.catalog_center_size_device(len(out["x"]), d[0].data_ptr(), d[1].data_ptr(),
                                        dz.data_ptr() if dz is not None else 0)
    assert got2 == got
