"""CPU tests of the 3-point class table: every class of the reference's module
(WrapCorr3, src/Corr3.cpp:4233-4262) is created with the zeta arrays of its ZetaData
(include/Corr3.h:581-720) and refused without them; combinations the reference does not
wrap and other binnings are refused.  tc_corr3_create is host code (no GPU needed)."""
import ctypes
import sys

import numpy as np
import pytest

CLASSES = ("NNN", "KKK", "GGG", "NNK", "NKN", "KNN", "NKK", "KNK", "KKN", "NNG", "NGN", "GNN",
           "NGG", "GNG", "GGN", "KKG", "KGK", "GKK", "KGG", "GKG", "GGK")


def nzeta(letters):
    """ZetaData<algo> arrays: 8 with three G's, 4 with two, none for NNN, else 2."""
    g = letters.count("G")
    return 8 if g == 3 else 4 if g == 2 else 0 if letters == "NNN" else 2


def make(T, letters, nz, bin_type=None, nb=4, mn=3):
    shape = (nb, nb, 2 * mn + 1)
    e = np.array([])
    zeta = [np.zeros(shape) for _ in range(nz)] + [e] * (8 - nz)
    rest = [np.zeros(shape) for _ in range(11)]
    bt = T.LogMultipole if bin_type is None else bin_type
    return getattr(T, letters + "Corr")(bt, 1.0, 10.0, nb, np.log(10.0) / nb, 0.1, 0.2, 0., 0.,
                                        mn, 0., 0., 0., 0., 0, 0., 0., -sys.float_info.max,
                                        sys.float_info.max, 0., 0., 0., *zeta, *rest)


@pytest.mark.parametrize("letters", CLASSES)
def test_class_created_with_its_zeta_arrays(letters):
    from treecorr_gb300 import _treecorr as T
    c = make(T, letters, nzeta(letters))
    assert c._h.value
    if nzeta(letters):
        with pytest.raises(ValueError):
            make(T, letters, nzeta(letters) - 1)


def test_unwrapped_combinations_and_binnings_refused():
    from treecorr_gb300 import _treecorr as T
    L = T.lib()
    shape = 4 * 4 * 7
    arrs = [np.zeros(shape) for _ in range(19)]
    ptrs = [a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for a in arrs]
    h = ctypes.c_void_p()
    kinds = {"N": 0, "K": 1, "G": 2, "Z": 3}
    for trio in ("NKG", "GKN", "KGN", "NNZ"):
        d = [kinds[x] for x in trio]
        rc = L.tc_corr3_create(*d, int(T.LogMultipole), 1.0, 10.0, 4, np.log(10.) / 4, 0.1, 0.2,
                               0., 0., 3, 0., 0., 0., 0., 0, 0., 0., -sys.float_info.max,
                               sys.float_info.max, 0., 0., 0., *ptrs, ctypes.byref(h))
        assert rc == T.TC_ERR_UNSUPPORTED, trio
    with pytest.raises(NotImplementedError):
        make(T, "GGG", 8, bin_type=T.LogRUV)

