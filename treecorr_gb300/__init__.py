"""treecorr_gb300 -- a GB300 (sm_103a) engine for TreeCorr's correlation hot path.

`treecorr_gb300._treecorr` is a drop-in for the reference's native module on the 2-point
path (ball-tree build, dual-tree traversal with the bin_slop rule, NN/KK/GG accumulation
with Log binning), backed by hand-written CUDA kernels in libtcgpu.so (C ABI:
include/tcgpu.h).
"""
from . import _treecorr  # noqa: F401

__all__ = ["_treecorr"]
