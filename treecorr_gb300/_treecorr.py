"""Drop-in for TreeCorr's native module ``_treecorr`` on the 2-point hot path.

Same class names, constructor signatures, methods and enum values as the reference's
pybind11 module (src/module.cpp:21-26; fields src/Field.cpp:610-703; correlations
src/Corr2.cpp:1132-1235), implemented over the C ABI of libtcgpu.so (include/tcgpu.h),
whose kernels run on the GPU.  TreeCorr's own Python layer can use it unchanged:

    import treecorr
    from treecorr_gb300 import _treecorr as gpu
    treecorr._treecorr = gpu            # or sys.modules['treecorr._treecorr'] = gpu

What is on the GPU path: N/K/G fields on Flat, Sphere and ThreeD coordinates, NN/KK/GG
correlations with Log binning, Euclidean (any coords) and Arc (spherical) metrics, split
methods Mean, Middle and Median.  Every other combination raises NotImplementedError --
there is no CPU fallback.  Errors from the library raise RuntimeError / ValueError (the
reference prints an Assert and continues).
"""
import ctypes
import enum
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_lib", "libtcgpu.so")

TC_OK, TC_ERR_ARG, TC_ERR_CUDA, TC_ERR_UNSUPPORTED, TC_ERR_DEVICE, TC_ERR_NOMEM = range(6)


class tc_stats(ctypes.Structure):
    _fields_ = [("cell_pairs", ctypes.c_int64), ("accepted", ctypes.c_int64),
                ("escalated", ctypes.c_int64), ("launches", ctypes.c_int64),
                ("build_ms", ctypes.c_double), ("traverse_ms", ctypes.c_double),
                ("learned", ctypes.c_int64), ("tiles", ctypes.c_int64),
                ("tile_pairs", ctypes.c_int64), ("tile_escalated", ctypes.c_int64),
                ("expand_ms", ctypes.c_double), ("tiles_ms", ctypes.c_double)]


CAT_MAXCOLS = 24


class tc_catalog_info(ctypes.Structure):
    _fields_ = [("nkeep", ctypes.c_int64), ("nobj", ctypes.c_int64), ("sumw", ctypes.c_double),
                ("nontrivial_w", ctypes.c_int), ("wpos_zero", ctypes.c_int64),
                ("wpos_conflicts", ctypes.c_int64),
                ("nan_counts", ctypes.c_int64 * (CAT_MAXCOLS + 2))]


_lib = None


def lib():
    """Load libtcgpu.so (built by treecorr_gb300.build); raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise ImportError("libtcgpu.so is not built: run `python -m treecorr_gb300.build` "
                              "(the GPU path has no CPU fallback)")
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        vp = ctypes.c_void_p
        i64 = ctypes.c_int64
        L.tc_field_create.restype = ctypes.c_int
        L.tc_field_create.argtypes = [ctypes.c_int, ctypes.c_int] + [dp] * 7 + [
            i64, ctypes.c_double, ctypes.c_double, ctypes.c_int, i64, ctypes.c_int,
            ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
        L.tc_field_create_device.restype = ctypes.c_int
        L.tc_field_create_device.argtypes = [ctypes.c_int, ctypes.c_int] + [vp] * 7 + [
            i64, ctypes.c_double, ctypes.c_double, ctypes.c_int, i64, ctypes.c_int,
            ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
        L.tc_field_free.restype = None
        L.tc_field_free.argtypes = [vp]
        L.tc_field_nobj.restype = i64
        L.tc_field_nobj.argtypes = [vp]
        L.tc_field_size.restype = ctypes.c_double
        L.tc_field_size.argtypes = [vp]
        L.tc_field_ntop.restype = i64
        L.tc_field_ntop.argtypes = [vp]
        L.tc_field_center.restype = ctypes.c_int
        L.tc_field_center.argtypes = [vp, dp]
        L.tc_field_dump.restype = i64
        L.tc_field_dump.argtypes = [vp, dp, ctypes.POINTER(ctypes.c_float),
                                    ctypes.POINTER(i64), ctypes.POINTER(ctypes.c_int32), i64]
        L.tc_corr2_create.restype = ctypes.c_int
        L.tc_corr2_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_int] + \
            [ctypes.c_double] * 8 + [dp] * 8 + [ctypes.POINTER(vp)]
        L.tc_corr2_free.restype = None
        L.tc_corr2_free.argtypes = [vp]
        L.tc_corr2_process_auto.restype = ctypes.c_int
        L.tc_corr2_process_auto.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.tc_corr2_process_cross.restype = ctypes.c_int
        L.tc_corr2_process_cross.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int]
        L.tc_corr2_trivially_zero.restype = ctypes.c_int
        L.tc_corr2_trivially_zero.argtypes = [vp, ctypes.c_int, ctypes.c_int] + \
            [ctypes.c_double] * 8 + [ctypes.POINTER(ctypes.c_int)]
        L.tc_corr2_stats.restype = ctypes.c_int
        L.tc_corr2_stats.argtypes = [vp, ctypes.POINTER(tc_stats)]
        i32p = ctypes.POINTER(ctypes.c_int32)
        L.tc_corr2_process_patches.restype = ctypes.c_int
        L.tc_corr2_process_patches.argtypes = [vp, ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int,
                                               ctypes.c_int, ctypes.c_int, i32p, i32p, dp,
                                               ctypes.POINTER(ctypes.c_int)]
        L.tc_jackknife_cov.restype = ctypes.c_int
        L.tc_jackknife_cov.argtypes = [dp, i32p, i32p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, dp, dp]
        L.tc_tcgen05_selftest.restype = ctypes.c_int
        L.tc_tcgen05_selftest.argtypes = [ctypes.POINTER(ctypes.c_float)] * 3 + [ctypes.c_int] * 2
        L.tc_generate_xyz.restype = ctypes.c_int
        L.tc_generate_xyz.argtypes = [dp, dp, dp, dp, dp, dp, i64]
        L.tc_generate_xyz_device.restype = ctypes.c_int
        L.tc_generate_xyz_device.argtypes = [vp, vp, vp, vp, vp, vp, i64]
        L.tc_catalog_finish.restype = ctypes.c_int
        L.tc_catalog_finish.argtypes = [i64, ctypes.c_int, ctypes.POINTER(dp), dp, dp,
                                        ctypes.POINTER(ctypes.c_int64), i64, ctypes.c_int,
                                        ctypes.c_int, ctypes.POINTER(tc_catalog_info)]
        L.tc_catalog_center_size.restype = ctypes.c_int
        L.tc_catalog_center_size.argtypes = [i64, dp, dp, dp, dp]
        L.tc_catalog_center_size_device.restype = ctypes.c_int
        L.tc_catalog_center_size_device.argtypes = [i64, vp, vp, vp, dp]
        L.tc_catalog_finish_device.restype = ctypes.c_int
        L.tc_catalog_finish_device.argtypes = [i64, ctypes.c_int, ctypes.POINTER(vp), vp, vp, vp,
                                               i64, ctypes.c_int, ctypes.c_int,
                                               ctypes.POINTER(tc_catalog_info)]
        fp = ctypes.POINTER(ctypes.c_float)
        L.tc_mlp_nparam.restype = ctypes.c_int
        L.tc_mlp_nparam.argtypes = []
        L.tc_corr2_set_tuning.restype = ctypes.c_int
        L.tc_corr2_set_tuning.argtypes = [vp, ctypes.c_int, i64]
        L.tc_corr2_autotune.restype = ctypes.c_int
        L.tc_corr2_autotune.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.c_double,
                                        ctypes.POINTER(ctypes.c_int), ctypes.POINTER(i64),
                                        ctypes.POINTER(ctypes.c_double)]
        L.tc_corr2_set_learned.restype = ctypes.c_int
        L.tc_corr2_set_learned.argtypes = [vp, fp, ctypes.c_double, ctypes.c_double]
        L.tc_learn_collect.restype = ctypes.c_int
        L.tc_learn_collect.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, i64, i64, fp, fp,
                                       ctypes.POINTER(i64)]
        L.tc_mlp_grad.restype = ctypes.c_int
        L.tc_mlp_grad.argtypes = [fp, fp, fp, i64, fp, fp]
        L.tc_mlp_infer.restype = ctypes.c_int
        L.tc_mlp_infer.argtypes = [fp, fp, i64, fp]
        L.tc_mlp_train.restype = ctypes.c_int
        L.tc_mlp_train.argtypes = [fp, fp, fp, i64, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                   ctypes.c_uint, fp]
        L.tc_set_omp_threads.restype = ctypes.c_int
        L.tc_set_omp_threads.argtypes = [ctypes.c_int]
        L.tc_get_omp_threads.restype = ctypes.c_int
        L.tc_get_omp_threads.argtypes = []
        L.tc_trim_memory.restype = ctypes.c_int
        L.tc_trim_memory.argtypes = []
        L.tc_set_deterministic.restype = ctypes.c_int
        L.tc_set_deterministic.argtypes = [ctypes.c_int]
        L.tc_get_deterministic.restype = ctypes.c_int
        L.tc_get_deterministic.argtypes = []
        L.tc_last_error.restype = ctypes.c_char_p
        L.tc_last_error.argtypes = []
        L.tc_corr3_create.restype = ctypes.c_int
        cd_, ci_ = ctypes.c_double, ctypes.c_int
        L.tc_corr3_create.argtypes = [ci_] * 4 + [cd_, cd_, ci_, cd_, cd_, cd_] + \
            [cd_, cd_, ci_, cd_, cd_] + [cd_, cd_, ci_, cd_, cd_] + [cd_] * 5 + [dp] * 19 + \
            [ctypes.POINTER(vp)]
        L.tc_corr3_free.restype = None
        L.tc_corr3_free.argtypes = [vp]
        L.tc_corr3_process_auto.restype = ctypes.c_int
        L.tc_corr3_process_auto.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.tc_corr3_process_cross12.restype = ctypes.c_int
        L.tc_corr3_process_cross12.argtypes = [vp, vp, vp] + [ctypes.c_int] * 4
        L.tc_corr3_process_cross21.restype = ctypes.c_int
        L.tc_corr3_process_cross21.argtypes = [vp, vp, vp] + [ctypes.c_int] * 4
        L.tc_corr3_process_cross.restype = ctypes.c_int
        L.tc_corr3_process_cross.argtypes = [vp, vp, vp, vp] + [ctypes.c_int] * 4
        L.tc_corr3_last_ms.restype = ctypes.c_double
        L.tc_corr3_last_ms.argtypes = [vp]
        L.tc_corr3_stats.restype = ctypes.c_int
        L.tc_corr3_stats.argtypes = [vp, ctypes.POINTER(i64)]
        lp64 = ctypes.POINTER(ctypes.c_int64)
        for nm in ("tc_kmeans_init_tree", "tc_kmeans_init_rand", "tc_kmeans_init_kmpp"):
            getattr(L, nm).restype = ctypes.c_int
            getattr(L, nm).argtypes = [vp, dp, ctypes.c_int, i64]
        L.tc_kmeans_run.restype = ctypes.c_int
        L.tc_kmeans_run.argtypes = [vp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_int]
        L.tc_kmeans_assign.restype = ctypes.c_int
        L.tc_kmeans_assign.argtypes = [vp, dp, ctypes.c_int, lp64, i64]
        L.tc_kmeans_iterations.restype = ctypes.c_int
        L.tc_kmeans_iterations.argtypes = [vp]
        L.tc_quick_assign.restype = ctypes.c_int
        L.tc_quick_assign.argtypes = [dp, ctypes.c_int, dp, dp, dp, i64, lp64]
        L.tc_select_patch.restype = ctypes.c_int
        L.tc_select_patch.argtypes = [ctypes.c_int, dp, ctypes.c_int, dp, dp, dp, i64, lp64]
        L.tc_quick_assign_device.restype = ctypes.c_int
        L.tc_quick_assign_device.argtypes = [dp, ctypes.c_int, vp, vp, vp, i64, vp]
        L.tc_select_patch_device.restype = ctypes.c_int
        L.tc_select_patch_device.argtypes = [ctypes.c_int, dp, ctypes.c_int, vp, vp, vp, i64, vp]
        L.tc_launch_count.restype = ctypes.c_longlong
        L.tc_launch_count.argtypes = []
        L.tc_stream.restype = ctypes.c_void_p
        L.tc_stream.argtypes = []
        _lib = L
    return _lib


def _check(rc):
    if rc == TC_OK:
        return
    msg = lib().tc_last_error().decode(errors="replace")
    if rc == TC_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if rc == TC_ERR_ARG:
        raise ValueError(msg)
    raise RuntimeError(f"tcgpu error {rc}: {msg}")


# ----------------------------------------------------------------------------------------
# Enums (values as in include/BinType.h:36, Position.h:24, Metric.h:29, Cell.h:26), exported
# at module level like pybind11's export_values (src/Corr2.cpp:1204-1234).

class BinType(enum.IntEnum):
    Log = 0
    Linear = 1
    TwoD = 2
    LogRUV = 3
    LogSAS = 4
    LogMultipole = 5


class Coord(enum.IntEnum):
    Flat = 1
    ThreeD = 2
    Sphere = 3


class Metric(enum.IntEnum):
    Euclidean = 1
    Rperp = 2
    Rlens = 3
    Arc = 4
    OldRperp = 5
    Periodic = 6


class SplitMethod(enum.IntEnum):
    Middle = 0
    Median = 1
    Mean = 2
    Random = 3


for _e in (BinType, Coord, Metric, SplitMethod):
    for _m in _e:
        globals()[_m.name] = _m
del _e, _m


def SetOMPThreads(num_threads):
    """SetOMPThreads (src/Corr2.cpp:995-1003): the GPU path has no host threads; returns 1."""
    return lib().tc_set_omp_threads(int(num_threads))


def GetOMPThreads():
    """GetOMPThreads (src/Corr2.cpp:1005-1011); returns 1."""
    return lib().tc_get_omp_threads()


def SetDeterministic(on=True):
    """Fixed-order 2-point expansion (default on): repeated process calls give bit-identical
    sums.  Returns the previous setting.  No reference counterpart."""
    return bool(lib().tc_set_deterministic(1 if on else 0))


def TrimMemory():
    """Returns the cached expansion buffers of freed corrs to the driver.  No reference
    counterpart."""
    _check(lib().tc_trim_memory())


def GetDeterministic():
    """Whether the fixed-order 2-point expansion is on.  No reference counterpart."""
    return bool(lib().tc_get_deterministic())


def _arr(a, n=None, name="array"):
    """Contiguous float64 copy/view, or None for an absent (empty) array."""
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.size == 0:
        return None
    if n is not None and a.size != n:
        raise ValueError(f"{name} has size {a.size}, expected {n}")
    return a


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


# ----------------------------------------------------------------------------------------
# Fields

class _FieldBase:
    _dkind = 0
    _coords = 1

    def _build(self, x, y, z, d1, d2, w, wpos, minsize, maxsize, sm, seed, brute, mintop,
               maxtop):
        x = _arr(x, name="x")
        n = 0 if x is None else x.size
        y = _arr(y, n, "y")
        z = _arr(z, n, "z")
        w = _arr(w, n, "w")
        wpos = _arr(wpos, n, "wpos")
        d1 = _arr(d1, n, "d1")
        d2 = _arr(d2, n, "d2")
        if self._coords == Coord.Flat:
            z = None
        self._keep = (x, y, z, d1, d2, w, wpos)
        h = ctypes.c_void_p()
        _check(lib().tc_field_create(self._dkind, int(self._coords), _ptr(x), _ptr(y), _ptr(z),
                                     _ptr(d1), _ptr(d2), _ptr(w), _ptr(wpos), n,
                                     float(minsize), float(maxsize), int(sm), int(seed),
                                     int(bool(brute)), int(mintop), int(maxtop),
                                     ctypes.byref(h)))
        self._h = h
        self._keep = None   # the library copied the data (src/Field.cpp:180-196)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            _lib.tc_field_free(h)
            self._h = None

    # BaseField methods (src/Field.cpp:624-634)
    def getNObj(self):
        return int(lib().tc_field_nobj(self._h))

    def getSize(self):
        return float(lib().tc_field_size(self._h))

    def getNTopLevel(self):
        r = lib().tc_field_ntop(self._h)
        if r < 0:
            _check(int(-r))
        return int(r)

    def countNear(self, *args):
        raise NotImplementedError("countNear is not on the GPU path")

    def getNear(self, *args):
        raise NotImplementedError("getNear is not on the GPU path")

    # k-means (src/Field.cpp:630-634 -> src/KMeans.cpp:851-888).  cenp is the caller's
    # (npatch, 2 or 3) float64 array, filled or refined in place like the reference's
    # py::array_t; pp receives the patch of every point.
    def _centers(self, cenp, npatch):
        dim = 2 if self._coords == Coord.Flat else 3
        if (not isinstance(cenp, np.ndarray) or cenp.dtype != np.float64 or
                not cenp.flags.c_contiguous or cenp.size != npatch * dim):
            raise ValueError(f"centers must be a contiguous float64 array of {npatch} x {dim}")
        return _ptr(cenp)

    def KMeansInitTree(self, cenp, npatch, seed):
        _check(lib().tc_kmeans_init_tree(self._h, self._centers(cenp, npatch), int(npatch), int(seed)))

    def KMeansInitRand(self, cenp, npatch, seed):
        _check(lib().tc_kmeans_init_rand(self._h, self._centers(cenp, npatch), int(npatch), int(seed)))

    def KMeansInitKMPP(self, cenp, npatch, seed):
        _check(lib().tc_kmeans_init_kmpp(self._h, self._centers(cenp, npatch), int(npatch), int(seed)))

    def KMeansRun(self, cenp, npatch, max_iter, tol, alt):
        _check(lib().tc_kmeans_run(self._h, self._centers(cenp, npatch), int(npatch),
                                   int(max_iter), float(tol), int(bool(alt))))

    def KMeansAssign(self, cenp, npatch, pp):
        if pp.dtype != np.int64 or not pp.flags.c_contiguous:
            raise ValueError("patches must be a contiguous int64 array")
        _check(lib().tc_kmeans_assign(self._h, self._centers(cenp, npatch), int(npatch),
                                      pp.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), pp.size))

    def kmeans_iterations(self):
        """Iterations run by the last KMeansRun (no reference counterpart)."""
        return int(lib().tc_kmeans_iterations(self._h))

    def _dump(self):
        """Canonical depth-first dump of the tree (tests only)."""
        cap = 2 * max(self.getNObj(), 1) + 2
        xyz = np.zeros((cap, 3))
        swd = np.zeros((cap, 4), dtype=np.float32)
        ns = np.zeros((cap, 2), dtype=np.int64)
        depth = np.zeros(cap, dtype=np.int32)
        cnt = lib().tc_field_dump(self._h, _ptr(xyz),
                                  swd.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                  ns.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                  depth.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), cap)
        if cnt < 0:
            _check(int(-cnt))
        return dict(x=xyz[:cnt, 0], y=xyz[:cnt, 1], z=xyz[:cnt, 2], size=swd[:cnt, 0],
                    w=swd[:cnt, 1], d1=swd[:cnt, 2], d2=swd[:cnt, 3], n=ns[:cnt, 0],
                    start=ns[:cnt, 1], depth=depth[:cnt])


def _field_class(name, dkind, coords):
    if dkind == 0:
        def __init__(self, x, y, z, w, wpos, minsize, maxsize, sm, seed, brute, mintop, maxtop):
            self._build(x, y, z, None, None, w, wpos, minsize, maxsize, sm, seed, brute,
                        mintop, maxtop)
    elif dkind == 1:
        def __init__(self, x, y, z, k, w, wpos, minsize, maxsize, sm, seed, brute, mintop,
                     maxtop):
            self._build(x, y, z, k, None, w, wpos, minsize, maxsize, sm, seed, brute, mintop,
                        maxtop)
    else:
        def __init__(self, x, y, z, g1, g2, w, wpos, minsize, maxsize, sm, seed, brute,
                     mintop, maxtop):
            self._build(x, y, z, g1, g2, w, wpos, minsize, maxsize, sm, seed, brute, mintop,
                        maxtop)
    return type(name, (_FieldBase,), {"__init__": __init__, "_dkind": dkind,
                                       "_coords": coords, "__module__": __name__})


# BuildNField / BuildKField / BuildZField / BuildVField / BuildGField / BuildTField /
# BuildQField (src/Field.cpp:430-560): {N,K,Z,V,G,T,Q}Field{Flat,Sphere,ThreeD}.
for _d, _k in (("N", 0), ("K", 1), ("G", 2), ("Z", 3), ("V", 4), ("T", 5), ("Q", 6)):
    for _c in ("Flat", "Sphere", "ThreeD"):
        globals()[_d + "Field" + _c] = _field_class(_d + "Field" + _c, _k, getattr(Coord, _c))
del _d, _k, _c


class DeviceField(_FieldBase):
    """A field built from catalog columns already resident on the GPU (no reference
    counterpart: the device-resident form of the N/K/G field constructors).  The columns are
    float64 device arrays given as integer pointers (e.g. torch.Tensor.data_ptr()) or
    0 for an absent column; they must stay alive until the constructor returns."""

    def __init__(self, dkind, coords, n, x, y, z, d1, d2, w, wpos, minsize, maxsize, sm, seed,
                 brute, mintop, maxtop):
        self._dkind = int(dkind)
        self._coords = int(coords)
        vp = ctypes.c_void_p
        h = vp()
        _check(lib().tc_field_create_device(self._dkind, self._coords, vp(x or None),
                                            vp(y or None), vp(z or None), vp(d1 or None),
                                            vp(d2 or None), vp(w or None), vp(wpos or None),
                                            int(n), float(minsize), float(maxsize), int(sm),
                                            int(seed), int(bool(brute)), int(mintop),
                                            int(maxtop), ctypes.byref(h)))
        self._h = h


def launch_count():
    """Kernels launched by libtcgpu.so since it was loaded."""
    return int(lib().tc_launch_count())


vp_t = ctypes.c_void_p

_CPW = {"simple": 0, "mean": 1, "match": 2}


def jackknife_cov(results, pairs, npatch, dkind, cross_patch_weight="simple"):
    """Jackknife design matrix and covariance on the GPU from processPatches results
    (_cov_jackknife, corr2base.py:2432-2445).  dkind: 1 (KK) or 2 (GG).  Returns (v, cov)."""
    results = np.ascontiguousarray(results, dtype=float)
    npair, _, nb = results.shape
    pi = np.ascontiguousarray([p[0] for p in pairs], dtype=np.int32)
    pj = np.ascontiguousarray([p[1] for p in pairs], dtype=np.int32)
    nstat = 2 if dkind == 2 else 1
    v = np.zeros((npatch, nstat * nb))
    cov = np.zeros((nstat * nb, nstat * nb))
    _check(lib().tc_jackknife_cov(_ptr(results), pi.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                  pj.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), npair, npatch,
                                  nb, int(dkind), _CPW[cross_patch_weight], _ptr(v), _ptr(cov)))
    return v, cov


def GenerateXYZ(x, y, z, ra, dec, r):
    """_treecorr.GenerateXYZ (src/KMeans.cpp:1013-1050): fills x, y, z in place from ra, dec
    (radians) and, unless r is empty, the distance r; computed on the GPU."""
    n = len(ra)
    for a in (x, y, z):
        if len(a) != n or a.dtype != np.float64 or not a.flags.c_contiguous:
            raise ValueError("x, y, z must be contiguous float64 arrays of len(ra)")
    ra = np.ascontiguousarray(ra, dtype=float)
    dec = np.ascontiguousarray(dec, dtype=float)
    if len(dec) != n or (len(r) not in (0, n)):
        raise ValueError("ra, dec and r must have the same length")
    rr = np.ascontiguousarray(r, dtype=float) if len(r) else None
    _check(lib().tc_generate_xyz(_ptr(x), _ptr(y), _ptr(z), _ptr(ra), _ptr(dec),
                                 _ptr(rr) if rr is not None else None, n))


# ----------------------------------------------------------------------------------------
# Catalog ingestion (treecorr/catalog.py:1343-1487; include/tcgpu.h tc_catalog_finish).

# The order of the reference's checkForNaN calls (treecorr/catalog.py:1407-1425).
CAT_COLUMNS = ("x", "y", "z", "ra", "dec", "r", "k", "z1", "z2", "v1", "v2", "g1", "g2",
               "t1", "t2", "q1", "q2")


def _cat_info(info, names, has_wpos):
    counts = {nm: int(info.nan_counts[i]) for i, nm in enumerate(names)}
    counts["w"] = int(info.nan_counts[len(names)])
    if has_wpos:
        counts["wpos"] = int(info.nan_counts[len(names) + 1])
    return dict(nkeep=int(info.nkeep), nobj=int(info.nobj), sumw=float(info.sumw),
                nontrivial_w=bool(info.nontrivial_w), wpos_zero=int(info.wpos_zero),
                wpos_conflicts=int(info.wpos_conflicts), nan_counts=counts)


def catalog_finish(cols, w=None, wpos=None, flag=None, ignore_flag=None, ok_flag=0,
                   keep_zero_weight=False):
    """Catalog._finish_input's column work on the GPU (flag -> w, NaN checks, wpos == 0,
    sumw, removal of zero-weight rows; treecorr/catalog.py:1343-1487).  cols: name -> array
    (names from CAT_COLUMNS).  Returns (cols, w, wpos, info) with the rows that remain; the
    inputs are not changed.  No reference counterpart in the native module: the reference
    does this in numpy inside Catalog."""
    names = [k for k in CAT_COLUMNS if k in cols]
    if len(names) != len(cols):
        raise ValueError("unknown column names: %s" % sorted(set(cols) - set(CAT_COLUMNS)))
    arrs = [np.array(cols[k], dtype=np.float64) for k in names]
    n = len(arrs[0]) if arrs else (len(w) if w is not None else 0)
    if any(len(a) != n for a in arrs):
        raise ValueError("columns of different lengths")
    w_given = w is not None
    wa = np.array(w, dtype=np.float64) if w_given else np.ones(n)
    wp = np.array(wpos, dtype=np.float64) if wpos is not None else None
    fl = np.ascontiguousarray(flag, dtype=np.int64) if flag is not None else None
    for a in ([wa] + ([wp] if wp is not None else []) + ([fl] if fl is not None else [])):
        if len(a) != n:
            raise ValueError("w, wpos and flag must have the columns' length")
    ignore = int(ignore_flag) if ignore_flag is not None else ~int(ok_flag)
    ptrs = (ctypes.POINTER(ctypes.c_double) * max(len(arrs), 1))(*[_ptr(a) for a in arrs])
    info = tc_catalog_info()
    _check(lib().tc_catalog_finish(
        n, len(arrs), ptrs, _ptr(wa), _ptr(wp) if wp is not None else None,
        fl.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)) if fl is not None else None,
        ignore, 1 if w_given else 0, 1 if keep_zero_weight else 0, ctypes.byref(info)))
    m = int(info.nkeep)
    out = {k: a[:m] for k, a in zip(names, arrs)}
    return out, wa[:m], (wp[:m] if wp is not None else None), _cat_info(info, names,
                                                                          wp is not None)


def catalog_center_size(x, y, z=None):
    """Catalog._get_center_size (treecorr/catalog.py:1330-1341) on the GPU: (mean x, mean y,
    mean z, largest distance from the mean).  No reference counterpart in the native module."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    zz = np.ascontiguousarray(z, dtype=np.float64) if z is not None else None
    out = np.zeros(4)
    _check(lib().tc_catalog_center_size(len(x), _ptr(x), _ptr(y), _ptr(zz), _ptr(out)))
    return tuple(float(v) for v in out)


def catalog_center_size_device(n, x_ptr, y_ptr, z_ptr=0):
    """catalog_center_size on device columns (integer addresses of float64 arrays)."""
    out = np.zeros(4)
    _check(lib().tc_catalog_center_size_device(int(n), ctypes.c_void_p(int(x_ptr)),
                                               ctypes.c_void_p(int(y_ptr)),
                                               ctypes.c_void_p(int(z_ptr)) if z_ptr else None,
                                               _ptr(out)))
    return tuple(float(v) for v in out)


def catalog_finish_device(n, col_ptrs, w_ptr, wpos_ptr=0, flag_ptr=0, ignore_flag=None,
                          ok_flag=0, w_given=True, keep_zero_weight=False, names=None):
    """catalog_finish on device columns (integer device addresses of float64 arrays, in
    CAT_COLUMNS order; flag: int64).  The columns are changed in place; info["nkeep"] rows
    remain.  No reference counterpart."""
    ptrs = (ctypes.c_void_p * max(len(col_ptrs), 1))(*[ctypes.c_void_p(int(p)) for p in col_ptrs])
    ignore = int(ignore_flag) if ignore_flag is not None else ~int(ok_flag)
    info = tc_catalog_info()
    _check(lib().tc_catalog_finish_device(
        int(n), len(col_ptrs), ptrs, ctypes.c_void_p(int(w_ptr)),
        ctypes.c_void_p(int(wpos_ptr)) if wpos_ptr else None,
        ctypes.c_void_p(int(flag_ptr)) if flag_ptr else None, ignore,
        1 if w_given else 0, 1 if keep_zero_weight else 0, ctypes.byref(info)))
    names = list(names) if names is not None else ["c%d" % i for i in range(len(col_ptrs))]
    return _cat_info(info, names, bool(wpos_ptr))


# ----------------------------------------------------------------------------------------
# Learned opening criterion (no reference counterpart; see include/tcgpu.h).

def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def tcgen05_selftest(a, b):
    """c = a @ b.T through the tcgen05 tensor cores (TF32, TMEM); a: 128 x k, b: n x k."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    c = np.zeros((a.shape[0], b.shape[0]), dtype=np.float32)
    _check(lib().tc_tcgen05_selftest(_fptr(a), _fptr(b), _fptr(c), b.shape[0], a.shape[1]))
    return c


def mlp_nparam():
    return int(lib().tc_mlp_nparam())


def mlp_grad(params, x, y):
    """Gradient and loss of the mean squared error of the network over (x, y), on the GPU."""
    params = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    g = np.zeros(mlp_nparam(), dtype=np.float32)
    loss = np.zeros(1, dtype=np.float32)
    _check(lib().tc_mlp_grad(_fptr(params), _fptr(x), _fptr(y), len(y), _fptr(g), _fptr(loss)))
    return g, float(loss[0])


def mlp_infer(params, x):
    """The traversal's FP16 tensor-core evaluation of the network over feature rows x."""
    params = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.zeros(len(x), dtype=np.float32)
    _check(lib().tc_mlp_infer(_fptr(params), _fptr(x), len(x), _fptr(y)))
    return y


def mlp_train(params, x, y, steps, batch=4096, lr=1e-3, seed=0):
    """Adam training on the GPU; returns (trained parameters, per-step loss)."""
    p = np.array(params, dtype=np.float32, copy=True)
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    loss = np.zeros(max(steps, 1), dtype=np.float32)
    _check(lib().tc_mlp_train(_fptr(p), _fptr(x), _fptr(y), len(y), int(steps), int(batch),
                              float(lr), int(seed), _fptr(loss)))
    return p, loss[:steps]


def stream_handle():
    """The cudaStream_t (as an int) on which libtcgpu.so launches its work."""
    return int(lib().tc_stream() or 0)


# ----------------------------------------------------------------------------------------
# Correlations

class BaseCorr2:
    """BaseCorr2 (src/Corr2.cpp:1168-1175): processAuto, processCross, triviallyZero."""
    _dkind = 0
    _dkind2 = None      # the second field's kind when it differs (NK, NG, ...)

    def __init__(self, bin_type, minsep, maxsep, nbins, binsize, b, a, minrpar, maxrpar, xp,
                 yp, zp, xi0, xi1, xi2, xi3, meanr, meanlogr, weight, npairs):
        # The outputs are aliased, never copied (BuildCorr2, src/Corr2.cpp:842-864).
        outs = []
        for name, arr in (("xi0", xi0), ("xi1", xi1), ("xi2", xi2), ("xi3", xi3),
                          ("meanr", meanr), ("meanlogr", meanlogr), ("weight", weight),
                          ("npairs", npairs)):
            if arr is None or arr.size == 0:
                outs.append(None)
                continue
            if arr.dtype != np.float64 or not arr.flags["C_CONTIGUOUS"] or \
                    not arr.flags["WRITEABLE"]:
                raise ValueError(f"{name} must be a writeable contiguous float64 array")
            if arr.size != int(nbins):
                raise ValueError(f"{name} has size {arr.size}, expected nbins={nbins}")
            outs.append(arr)
        self._outs = outs
        self._nbins = int(nbins)
        h = ctypes.c_void_p()
        d2 = self._dkind if self._dkind2 is None else self._dkind2
        _check(lib().tc_corr2_create(self._dkind, d2, int(bin_type), float(minsep),
                                     float(maxsep), int(nbins), float(binsize), float(b),
                                     float(a), float(minrpar), float(maxrpar), float(xp),
                                     float(yp), float(zp), *[_ptr(o) for o in outs],
                                     ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            _lib.tc_corr2_free(h)
            self._h = None

    def processAuto(self, field, dots, quick, metric):
        _check(lib().tc_corr2_process_auto(self._h, field._h, int(bool(dots)), int(bool(quick)),
                                           int(metric)))

    def processCross(self, field1, field2, dots, quick, metric):
        _check(lib().tc_corr2_process_cross(self._h, field1._h, field2._h, int(bool(dots)),
                                            int(bool(quick)), int(metric)))

    def triviallyZero(self, metric, coords, x1, y1, z1, s1, x2, y2, z2, s2):
        out = ctypes.c_int(0)
        _check(lib().tc_corr2_trivially_zero(self._h, int(metric), int(coords), float(x1),
                                             float(y1), float(z1), float(s1), float(x2),
                                             float(y2), float(z2), float(s2), ctypes.byref(out)))
        return int(out.value)

    def samplePairs(self, *args):
        raise NotImplementedError("samplePairs is not on the GPU path")

    def processPatches(self, fields, metric, quick=False):
        """Every patch-pair correlation of the patch fields in one GPU expansion (the Python
        loop of corr2base.py:929-950).  Returns (pairs, results): pairs [(i, j)], i <= j, and
        results [npair, 8, nbins] = weight, meanr, meanlogr, xi0..xi3, npairs for each pair
        (raw sums).  No reference counterpart in the native module."""
        n = len(fields)
        arr = (vp_t * n)(*[f._h for f in fields])
        maxp = n * (n + 1) // 2
        nb = self._nbins
        pi = np.zeros(maxp, dtype=np.int32)
        pj = np.zeros(maxp, dtype=np.int32)
        res = np.zeros((maxp, 8, nb))
        npair = ctypes.c_int(0)
        _check(lib().tc_corr2_process_patches(
            self._h, arr, n, int(metric), int(bool(quick)), maxp,
            pi.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
            pj.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _ptr(res), ctypes.byref(npair)))
        k = npair.value
        return list(zip(pi[:k].tolist(), pj[:k].tolist())), res[:k].copy()

    def setTuning(self, tile_leaf=0, chunk=0):
        """Tile leaf size and expansion chunk of the following process calls (0 = defaults).
        No reference counterpart."""
        _check(lib().tc_corr2_set_tuning(self._h, int(tile_leaf), int(chunk)))

    def autotune(self, field1, field2=None, metric=None, frac=0.05):
        """Times this correlation on a frac of its top-level pairs for several tile leaf sizes
        and expansion chunks and keeps the fastest (cached per configuration for the process;
        the output arrays are not touched).  Returns {tile_leaf, chunk, ms}.  No reference
        counterpart."""
        leaf, ch, ms = ctypes.c_int(0), ctypes.c_int64(0), ctypes.c_double(0.)
        m = int(metric if metric is not None else Metric.Euclidean)
        _check(lib().tc_corr2_autotune(self._h, field1._h, field2._h if field2 is not None else None,
                                       m, float(frac), ctypes.byref(leaf), ctypes.byref(ch),
                                       ctypes.byref(ms)))
        return {"tile_leaf": leaf.value, "chunk": ch.value, "ms": ms.value}

    def setLearned(self, params=None, threshold=-2.0, cand_factor=4.0):
        """Use the learned opening criterion (params: tc_mlp_nparam() floats) in the following
        process calls, or the bin_slop rule alone (params=None).  No reference counterpart."""
        if params is None:
            _check(lib().tc_corr2_set_learned(self._h, None, 0.0, 0.0))
            self._mlp = None
            return
        self._mlp = np.ascontiguousarray(params, dtype=np.float32)
        _check(lib().tc_corr2_set_learned(self._h, _fptr(self._mlp), float(threshold),
                                          float(cand_factor)))

    def learnCollect(self, field, metric, sample_mod=16, max_samples=1 << 20,
                     max_point_pairs=1 << 16):
        """processAuto with the bin_slop rule, sampling training pairs for the learned
        criterion; returns (features [n, 5], targets [n]) (NaN targets: too many points)."""
        f = np.zeros((max_samples, 5), dtype=np.float32)
        t = np.zeros(max_samples, dtype=np.float32)
        n = ctypes.c_int64(0)
        _check(lib().tc_learn_collect(self._h, field._h, int(metric), int(sample_mod),
                                      int(max_samples), int(max_point_pairs), _fptr(f), _fptr(t),
                                      ctypes.byref(n)))
        return f[:n.value].copy(), t[:n.value].copy()

    def stats(self):
        """Counters of the last process call (no reference counterpart)."""
        s = tc_stats()
        _check(lib().tc_corr2_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in tc_stats._fields_}


# The 2-point classes of src/Corr2.cpp:1204-1232 (WrapCorr2<D1,D2>): NN, NK, KK and NX, KX,
# XX for the complex kinds X = Z, V, G, T, Q (data kind numbers of include/tcgpu.h).
_DKIND = {"N": 0, "K": 1, "G": 2, "Z": 3, "V": 4, "T": 5, "Q": 6}


def _corr2_class(d1, d2):
    return type(d1 + d2 + "Corr", (BaseCorr2,),
                {"_dkind": _DKIND[d1], "_dkind2": _DKIND[d2], "__module__": __name__})


NNCorr = _corr2_class("N", "N")
NKCorr = _corr2_class("N", "K")
KKCorr = _corr2_class("K", "K")
for _x in "ZVGTQ":
    for _a in ("N", "K", _x):
        globals()[_a + _x + "Corr"] = _corr2_class(_a, _x)
del _x, _a


class BaseCorr3:
    """BaseCorr3 (src/Corr3.cpp:4187-4201): processAuto, processCross12, processCross21 and
    processCross with LogMultipole binning."""

    def processAuto(self, field, dots, quick, metric):
        _check(lib().tc_corr3_process_auto(self._h, field._h, int(bool(dots)), int(bool(quick)),
                                           int(metric)))

    def processCross12(self, field1, field2, ordered, dots, quick, metric):
        """One vertex from field1, two from field2 (ProcessCross12c, src/Corr3.cpp:3730-3768)."""
        _check(lib().tc_corr3_process_cross12(self._h, field1._h, field2._h, int(ordered),
                                              int(bool(dots)), int(bool(quick)), int(metric)))

    def processCross21(self, field1, field2, ordered, dots, quick, metric):
        """Two vertices from field1, one from field2 (ProcessCross21c, src/Corr3.cpp:3831-3868)."""
        _check(lib().tc_corr3_process_cross21(self._h, field1._h, field2._h, int(ordered),
                                              int(bool(dots)), int(bool(quick)), int(metric)))

    def processCross(self, field1, field2, field3, ordered, dots, quick, metric):
        """One vertex from each field (ProcessCrossc, src/Corr3.cpp:3938-3976)."""
        _check(lib().tc_corr3_process_cross(self._h, field1._h, field2._h, field3._h,
                                            int(ordered), int(bool(dots)), int(bool(quick)),
                                            int(metric)))

    def triviallyZero(self, *args):
        raise NotImplementedError("triviallyZero for 3-point is not on the GPU path")

    def last_ms(self):
        """Device time of the last processAuto in ms (no reference counterpart)."""
        return float(lib().tc_corr3_last_ms(self._h))

    def stats(self):
        """Counters of the last process call (no reference counterpart): vertex records
        contracted in batches, records contracted in place, finish/contract waves."""
        out = (ctypes.c_int64 * 3)()
        _check(lib().tc_corr3_stats(self._h, out))
        return {"records": int(out[0]), "in_place": int(out[1]), "waves": int(out[2])}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            _lib.tc_corr3_free(h)
            self._h = None


class GGGCorr(BaseCorr3):
    """GGGCorr (BuildCorr3, src/Corr3.cpp:3599-3645): outputs aliased, accumulated."""
    _dkind = 2

    def __init__(self, bin_type, minsep, maxsep, nbins, binsize, b, a, minu, maxu, nubins,
                 ubinsize, bu, minv, maxv, nvbins, vbinsize, bv, minrpar, maxrpar, xp, yp, zp,
                 zeta0, zeta1, zeta2, zeta3, zeta4, zeta5, zeta6, zeta7, meand1, meanlogd1,
                 meand2, meanlogd2, meand3, meanlogd3, meanu, meanv, weight, weight_im, ntri):
        arrs = [zeta0, zeta1, zeta2, zeta3, zeta4, zeta5, zeta6, zeta7, meand1, meanlogd1,
                meand2, meanlogd2, meand3, meanlogd3, meanu, meanv, weight, weight_im, ntri]
        size = int(nbins) * int(nbins) * (2 * int(nubins) + 1)
        for a_ in arrs:
            if a_ is None or a_.size == 0:
                continue
            if a_.dtype != np.float64 or not a_.flags["C_CONTIGUOUS"] or a_.size != size:
                raise ValueError("3-point outputs must be contiguous float64 arrays of "
                                 "nbins*nbins*(2*max_n+1) entries")
        self._outs = arrs
        h = ctypes.c_void_p()
        d1, d2 = self._dkind, getattr(self, "_dkind2", self._dkind)
        d3 = getattr(self, "_dkind3", d2)
        _check(lib().tc_corr3_create(d1, d2, d3, int(bin_type), float(minsep), float(maxsep),
                                     int(nbins), float(binsize), float(b), float(a), float(minu),
                                     float(maxu), int(nubins), float(ubinsize), float(bu),
                                     float(minv), float(maxv), int(nvbins), float(vbinsize),
                                     float(bv), float(minrpar), float(maxrpar), float(xp),
                                     float(yp), float(zp),
                                     *[_ptr(a_ if a_ is not None and a_.size else None)
                                       for a_ in arrs], ctypes.byref(h)))
        self._h = h


class NNNCorr(GGGCorr):
    """NNNCorr (src/Corr3.cpp:4237) with LogMultipole binning: weight, weight_im, ntri and
    the mean distances (the zeta arrays are empty for NNN)."""
    _dkind = 0


class KKKCorr(GGGCorr):
    """KKKCorr (src/Corr3.cpp:4238) with LogMultipole binning: zeta0, zeta1 = zeta (real,
    imaginary), weight, weight_im, ntri and the mean distances."""
    _dkind = 1


class NKKCorr(GGGCorr):
    """NKKCorr (src/Corr3.cpp:4245) with LogMultipole binning, processCross12 only (an N
    vertex and two K vertices): zeta0, zeta1 = zeta (real, imaginary), weight, weight_im,
    ntri and the mean distances."""
    _dkind = 0
    _dkind2 = 1


class KNNCorr(GGGCorr):
    """KNNCorr (src/Corr3.cpp:4243) with LogMultipole binning, processCross12 only (a K
    vertex and two N vertices): zeta0, zeta1 = zeta (real, imaginary), weight, weight_im,
    ntri and the mean distances."""
    _dkind = 1
    _dkind2 = 0


class NGGCorr(GGGCorr):
    """NGGCorr (src/Corr3.cpp:4253) with LogMultipole binning, processCross12 only (an N
    vertex and two G vertices): zeta0..3 = gam0r, gam0i, gam1r, gam1i; weight, weight_im,
    ntri and the mean distances."""
    _dkind = 0
    _dkind2 = 2


class KGGCorr(GGGCorr):
    """KGGCorr (src/Corr3.cpp:4261) with LogMultipole binning, processCross12 only (a K
    vertex and two G vertices): zeta0..3 = gam0r, gam0i, gam1r, gam1i; weight, weight_im,
    ntri and the mean distances."""
    _dkind = 1
    _dkind2 = 2


class GNNCorr(GGGCorr):
    """GNNCorr (src/Corr3.cpp:4251) with LogMultipole binning, processCross12 only (a G
    vertex and two N vertices): zeta0, zeta1 = zeta (real, imaginary), weight, weight_im,
    ntri and the mean distances."""
    _dkind = 2
    _dkind2 = 0


class GKKCorr(GGGCorr):
    """GKKCorr (src/Corr3.cpp:4259) with LogMultipole binning, processCross12 only (a G
    vertex and two K vertices): zeta0, zeta1 = zeta (real, imaginary), weight, weight_im,
    ntri and the mean distances."""
    _dkind = 2
    _dkind2 = 1


def _corr3_class(name):
    """The mixed classes whose vertices 2 and 3 differ (WrapCorr3, src/Corr3.cpp:4240-4262):
    processCross21 / processCross only."""
    return type(name + "Corr", (GGGCorr,),
                {"_dkind": _DKIND[name[0]], "_dkind2": _DKIND[name[1]],
                 "_dkind3": _DKIND[name[2]], "__module__": __name__,
                 "__doc__": f"{name}Corr (src/Corr3.cpp WrapCorr3) with LogMultipole binning."})


for _n in ("NNK", "NKN", "KNK", "KKN", "NNG", "NGN", "GNG", "GGN", "KKG", "KGK", "GKG", "GGK"):
    globals()[_n + "Corr"] = _corr3_class(_n)
del _n




def _assign_args(cenp, npatch, xp, yp, zp, out):
    n = len(xp)
    x = np.ascontiguousarray(xp, dtype=np.float64)
    y = np.ascontiguousarray(yp, dtype=np.float64)
    z = np.ascontiguousarray(zp, dtype=np.float64) if len(zp) else None
    dim = 3 if z is not None else 2
    if len(y) != n or (z is not None and len(z) != n) or len(out) != n:
        raise ValueError("x, y, z and the output must have the same length")
    cen = np.ascontiguousarray(cenp, dtype=np.float64)
    if cen.size != npatch * dim:
        raise ValueError(f"centers must have {npatch} x {dim} entries")
    if out.dtype != np.int64 or not out.flags.c_contiguous:
        raise ValueError("the output must be a contiguous int64 array")
    return cen, x, y, z, n


def QuickAssign(cenp, npatch, xp, yp, zp, pp):
    """QuickAssign (src/KMeans.cpp:890-942): pp[i] = the nearest centre of point i; an empty
    zp selects the 2-d form.  Computed on the GPU."""
    cen, x, y, z, n = _assign_args(cenp, npatch, xp, yp, zp, pp)
    _check(lib().tc_quick_assign(_ptr(cen), int(npatch), _ptr(x), _ptr(y), _ptr(z), n,
                                 pp.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))


def SelectPatch(patch, cenp, npatch, xp, yp, zp, usep):
    """SelectPatch (src/KMeans.cpp:944-1011): usep[i] = 1 when patch is the nearest centre
    of point i, else 0.  Computed on the GPU."""
    cen, x, y, z, n = _assign_args(cenp, npatch, xp, yp, zp, usep)
    _check(lib().tc_select_patch(int(patch), _ptr(cen), int(npatch), _ptr(x), _ptr(y), _ptr(z),
                                 n, usep.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
