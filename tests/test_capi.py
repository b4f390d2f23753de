"""CPU tests of the C ABI library: it loads without a GPU and exports every function that
include/tcgpu.h declares.  No compute call is made here."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "tcgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w\s\*]*?\b(tc_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from treecorr_gb300 import build as tb
    path = tb.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("tc_field_create", "tc_field_create_device", "tc_field_free", "tc_field_ntop",
                 "tc_corr2_create", "tc_corr2_process_auto", "tc_corr2_process_cross",
                 "tc_corr2_trivially_zero", "tc_last_error", "tc_corr2_process_auto_noalloc"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_mirror_matches_reference_names():
    """The mirror exports the reference module's names on this path, with its enum values
    (src/Corr2.cpp:1204-1234, include/Position.h:24, Metric.h:29, Cell.h:26, BinType.h:36)."""
    from treecorr_gb300 import _treecorr as T
    for d in "NKZVGTQ":
        for c in ("Flat", "Sphere", "ThreeD"):
            assert hasattr(T, d + "Field" + c), d + "Field" + c
    classes = ["NN", "NK", "KK"] + [a + x for x in "ZVGTQ" for a in ("N", "K", x)]
    for n in [c + "Corr" for c in classes] + ["BaseCorr2", "GGGCorr", "SetOMPThreads",
                                               "GetOMPThreads", "QuickAssign", "SelectPatch",
                                               "GenerateXYZ"]:
        assert hasattr(T, n), n
    assert (int(T.Flat), int(T.ThreeD), int(T.Sphere)) == (1, 2, 3)
    assert (int(T.Euclidean), int(T.Rperp), int(T.Rlens), int(T.Arc), int(T.OldRperp),
            int(T.Periodic)) == (1, 2, 3, 4, 5, 6)
    assert (int(T.Middle), int(T.Median), int(T.Mean), int(T.Random)) == (0, 1, 2, 3)
    assert (int(T.Log), int(T.Linear), int(T.TwoD), int(T.LogRUV), int(T.LogSAS),
            int(T.LogMultipole)) == (0, 1, 2, 3, 4, 5)
    # All 21 3-point classes of the reference's module are there.
    for n in ("NNN", "KKK", "GGG", "NNK", "NKN", "KNN", "NKK", "KNK", "KKN", "NNG", "NGN",
              "GNN", "NGG", "GNG", "GGN", "KKG", "KGK", "GKK", "KGG", "GKG", "GGK"):
        assert isinstance(getattr(T, n + "Corr"), type), n
