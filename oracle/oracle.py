"""ctypes front end of the CPU oracle (oracle/tc_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline / --impl reference legs, as the checker.  The product (treecorr_gb300) never
imports this module.

The oracle restates the reference TreeCorr algorithm for the 2-point hot path; its parity
with the reference C++ is pinned by the fixtures in tests/golden/.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")

DTYPES = {"N": 0, "K": 1, "G": 2, "Z": 3, "V": 4, "T": 5, "Q": 6}
COORDS = {"flat": 1, "3d": 2, "spherical": 3}
METRICS = {"Euclidean": 1, "Arc": 4}
SPLITS = {"middle": 0, "median": 1, "mean": 2}

_lib = None


def build():
    """Compile the oracle with its Makefile (seconds)."""
    subprocess.check_call(["make", "-s", "-f", os.path.join("oracle", "Makefile")], cwd=_ROOT)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        L.orc_field_build.restype = ctypes.c_void_p
        L.orc_field_build.argtypes = [ctypes.c_int, ctypes.c_int] + [dp] * 7 + [
            ctypes.c_long, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
            ctypes.c_int, ctypes.c_int]
        L.orc_field_free.argtypes = [ctypes.c_void_p]
        L.orc_field_ntop.restype = ctypes.c_long
        L.orc_field_ntop.argtypes = [ctypes.c_void_p]
        L.orc_field_center.argtypes = [ctypes.c_void_p, dp]
        L.orc_field_dump.restype = ctypes.c_long
        L.orc_field_dump.argtypes = [ctypes.c_void_p, dp, ctypes.POINTER(ctypes.c_float),
                                     ctypes.POINTER(ctypes.c_long),
                                     ctypes.POINTER(ctypes.c_int), ctypes.c_long]
        L.orc_field_order.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_long)]
        L.orc_corr2_process.restype = ctypes.c_int
        L.orc_corr2_process.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int] + [dp] * 8
        L.orc_corr2_process_rows.restype = ctypes.c_int
        L.orc_corr2_process_rows.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                             ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                             ctypes.c_void_p, ctypes.c_long, ctypes.c_long,
                                             ctypes.c_int] + [dp] * 8
        L.orc_corr3_multipole_auto.restype = ctypes.c_int
        L.orc_corr3_multipole_auto.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                               ctypes.c_void_p, ctypes.c_int,
                                               ctypes.POINTER(dp)] + [dp] * 7
        L.orc_corr3_multipole_cross12.restype = ctypes.c_int
        L.orc_corr3_multipole_cross12.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                                  ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                                  ctypes.c_int, ctypes.POINTER(dp)] + [dp] * 7
        L.orc_corr3_multipole_cross3.restype = ctypes.c_int
        L.orc_corr3_multipole_cross3.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                 ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                                 ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                                 ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                 ctypes.c_int, ctypes.POINTER(dp)] + [dp] * 7
        L.orc_last_accepted.restype = ctypes.c_longlong
        L.orc_last_accepted.argtypes = []
        L.orc_max_threads.restype = ctypes.c_int
        lp = ctypes.POINTER(ctypes.c_long)
        for nm in ("orc_kmeans_init_tree", "orc_kmeans_init_rand", "orc_kmeans_init_kmpp"):
            getattr(L, nm).restype = ctypes.c_int
            getattr(L, nm).argtypes = [ctypes.c_void_p, dp, ctypes.c_int, ctypes.c_longlong]
        L.orc_kmeans_run.restype = ctypes.c_int
        L.orc_kmeans_run.argtypes = [ctypes.c_void_p, dp, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_double, ctypes.c_int]
        L.orc_kmeans_assign.restype = ctypes.c_int
        L.orc_kmeans_assign.argtypes = [ctypes.c_void_p, dp, ctypes.c_int, lp]
        L.orc_quick_assign.argtypes = [dp, ctypes.c_int, dp, dp, dp, ctypes.c_long, lp]
        L.orc_select_patch.argtypes = [ctypes.c_int, dp, ctypes.c_int, dp, dp, dp,
                                       ctypes.c_long, lp]
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class OracleField:
    """A field built by the oracle; mirrors the arguments of _treecorr.{N,K,G}Field*."""

    def __init__(self, dtype, coords, x, y, z=None, d1=None, d2=None, w=None, wpos=None,
                 min_size=0.0, max_size=np.inf, split_method="mean", brute=False,
                 min_top=3, max_top=10):
        L = lib()
        self._keep = [np.ascontiguousarray(a, dtype=float) if a is not None else None
                      for a in (x, y, z, d1, d2, w, wpos)]
        x, y, z, d1, d2, w, wpos = self._keep
        self.n = len(x)
        self.coords = coords
        self.h = L.orc_field_build(DTYPES[dtype], COORDS[coords], _p(x), _p(y), _p(z),
                                   _p(d1), _p(d2), _p(w), _p(wpos), self.n,
                                   float(min_size), float(max_size), SPLITS[split_method],
                                   int(bool(brute)), int(min_top), int(max_top))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_field_free(self.h)
            self.h = None

    def ntop(self):
        return lib().orc_field_ntop(self.h)

    def center(self):
        out = np.zeros(4)
        lib().orc_field_center(self.h, _p(out))
        return out

    def dump(self):
        """Canonical depth-first dump: dict of arrays (x,y,z,size,w,d1,d2,n,start,depth)."""
        L = lib()
        cap = 2 * self.n + 2
        xyz = np.zeros((cap, 3))
        swd = np.zeros((cap, 4), dtype=np.float32)
        ns = np.zeros((cap, 2), dtype=np.int64)
        depth = np.zeros(cap, dtype=np.int32)
        cnt = L.orc_field_dump(self.h, _p(xyz), swd.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                               ns.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                               depth.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), cap)
        return dict(x=xyz[:cnt, 0], y=xyz[:cnt, 1], z=xyz[:cnt, 2], size=swd[:cnt, 0],
                    w=swd[:cnt, 1], d1=swd[:cnt, 2], d2=swd[:cnt, 3], n=ns[:cnt, 0],
                    start=ns[:cnt, 1], depth=depth[:cnt])

    # k-means (src/KMeans.cpp) on the oracle's tree; centers: (npatch, 2 or 3) float64.
    def kmeans_init(self, npatch, init="tree", seed=1):
        dim = 2 if self.coords == "flat" else 3
        cen = np.zeros((npatch, dim))
        fn = {"tree": "orc_kmeans_init_tree", "random": "orc_kmeans_init_rand",
              "kmeans++": "orc_kmeans_init_kmpp"}[init]
        rc = getattr(lib(), fn)(self.h, _p(cen), int(npatch), int(seed))
        if rc:
            raise RuntimeError("oracle k-means init failed")
        return cen

    def kmeans_run(self, centers, max_iter=200, tol=1e-5, alt=False):
        """Refines a copy of centers; returns (centers, iterations)."""
        cen = np.ascontiguousarray(centers, dtype=float).copy()
        it = lib().orc_kmeans_run(self.h, _p(cen), cen.shape[0], int(max_iter), float(tol),
                                  int(bool(alt)))
        return cen, it

    def kmeans_assign(self, centers):
        cen = np.ascontiguousarray(centers, dtype=float)
        out = np.empty(self.n, dtype=np.int64)
        lib().orc_kmeans_assign(self.h, _p(cen), cen.shape[0],
                                out.ctypes.data_as(ctypes.POINTER(ctypes.c_long)))
        return out

    def order(self):
        out = np.zeros(self.n, dtype=np.int64)
        lib().orc_field_order(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_long)))
        return out


def bin_setup(min_sep, max_sep, nbins, bin_slop=None, angle_slop=0.1):
    """Log binning + slop as the reference's Python layer derives them
    (treecorr/corr2base.py:420-443, 519-523)."""
    bin_size = np.log(max_sep / min_sep) / nbins
    max_good_slop = 0.1 / bin_size
    if bin_slop is None or bin_slop < 0:
        bin_slop = min(max_good_slop, 1.0)
    b = bin_size * bin_slop
    return dict(min_sep=float(min_sep), max_sep=float(max_sep), nbins=int(nbins),
                bin_size=float(bin_size), b=float(b), a=float(angle_slop))


def minmax_size(metric, bins):
    """Corr2._get_minmax_size for Log binning (treecorr/corr2base.py:1595-1625)."""
    if metric == "Euclidean":
        b1 = min(bins["a"], bins["b"])
        return bins["min_sep"] * b1 / (2. + 3. * b1), bins["max_sep"] * b1
    return 0.0, 0.0


def dpair(dtype):
    """The correlation's two data kinds ("GG" or "G" for GG, "NG", ...) as d1 * 16 + d2."""
    d1, d2 = (dtype[0], dtype[-1])
    return DTYPES[d1] * 16 + DTYPES[d2]


def process(dtype, metric, bins, f1, f2=None, quick=False, nthreads=0, rows=None):
    """Run the oracle's 2-point process; returns a dict of the 8 accumulated arrays."""
    nb = bins["nbins"]
    out = {k: np.zeros(nb) for k in ("xi0", "xi1", "xi2", "xi3", "meanr", "meanlogr",
                                      "weight", "npairs")}
    args = [dpair(dtype), METRICS[metric], int(bool(quick)), bins["min_sep"], bins["max_sep"],
            nb, bins["bin_size"], bins["b"], bins["a"]]
    ptrs = [_p(out[k]) for k in ("xi0", "xi1", "xi2", "xi3", "meanr", "meanlogr", "weight",
                                 "npairs")]
    L = lib()
    if rows is None:
        L.orc_corr2_process(*args, f1.h, f2.h if f2 is not None else None, int(nthreads), *ptrs)
    else:
        L.orc_corr2_process_rows(*args, f1.h, int(rows[0]), int(rows[1]), int(nthreads), *ptrs)
    out["_accepted"] = int(L.orc_last_accepted())
    return out


def max_threads():
    return lib().orc_max_threads()


MP_KEYS = ("gam0r", "gam0i", "gam1r", "gam1i", "gam2r", "gam2i", "gam3r", "gam3i",
           "meand2", "meanlogd2", "meand3", "meanlogd3", "weight", "weight_im", "ntri")


def multipole(metric, bins, max_n, f, quick=False, nthreads=0, f2=None, mode=0):
    """The oracle's GGG LogMultipole auto-correlation, or with f2 the cross12 one (vertex 1
    from f, vertices 2 and 3 from f2); dict of (nbins, nbins, 2*max_n+1) arrays (zeta0..7
    as gam0r..gam3i, meand2/3, meanlogd2/3, weight, weight_im, ntri).  mode 1 is the
    NGG / KGG form (vertex 1 a K field whose k is 1 or k): gam0 and gam2 are then their
    zeta0 and zeta1; mode 2 the GNN / GKK form (f2 such a K field): gam0 is their zeta;
    mode 3 the KKK / NKK / KNN form (f and f2 such K fields): gam0 is their zeta."""
    nb = bins["nbins"]
    shape = (nb, nb, 2 * max_n + 1)
    out = {k: np.zeros(shape) for k in MP_KEYS}
    gam = (ctypes.POINTER(ctypes.c_double) * 8)(*[_p(out[k]) for k in MP_KEYS[:8]])
    head = (METRICS[metric], int(bool(quick)), bins["min_sep"], bins["max_sep"], nb,
            bins["bin_size"], bins["b"], bins["a"], int(max_n))
    tail = [_p(out[k]) for k in MP_KEYS[8:]]
    if f2 is None:
        rc = lib().orc_corr3_multipole_auto(*head, f.h, int(nthreads), gam, *tail)
    else:
        rc = lib().orc_corr3_multipole_cross12(*head, f.h, f2.h, int(mode), int(nthreads), gam,
                                               *tail)
    if rc:
        raise ValueError("multipole needs G fields in one coordinate system")
    return out


def multipole3(metric, bins, max_n, f1, f2, f3, ordered, quick=False, nthreads=0, mode=0,
               out=None):
    """The oracle's three-field LogMultipole (vertex 1 from f1, 2 from f2, 3 from f3,
    ordered 1 or 4), accumulated into out (a dict as multipole returns) when given.  mode
    bits: 1 vertex 1, 2 vertex 2, 4 vertex 3 given as a K field whose k is 1 (N) or k (K)
    (a real payload)."""
    nb = bins["nbins"]
    shape = (nb, nb, 2 * max_n + 1)
    if out is None:
        out = {k: np.zeros(shape) for k in MP_KEYS}
    gam = (ctypes.POINTER(ctypes.c_double) * 8)(*[_p(out[k]) for k in MP_KEYS[:8]])
    rc = lib().orc_corr3_multipole_cross3(
        METRICS[metric], int(bool(quick)), bins["min_sep"], bins["max_sep"], nb,
        bins["bin_size"], bins["b"], bins["a"], int(max_n), f1.h, f2.h, f3.h, int(ordered),
        int(mode), int(nthreads), gam, *[_p(out[k]) for k in MP_KEYS[8:]])
    if rc:
        raise ValueError("multipole3: fields, coordinates or ordered not supported")
    return out


def quick_assign(centers, x, y, z=None):
    """QuickAssign (src/KMeans.cpp:890-942) restated; z None selects the 2-d form."""
    cen = np.ascontiguousarray(centers, dtype=float)
    x = np.ascontiguousarray(x, dtype=float)
    y = np.ascontiguousarray(y, dtype=float)
    z = None if z is None else np.ascontiguousarray(z, dtype=float)
    out = np.empty(len(x), dtype=np.int64)
    lib().orc_quick_assign(_p(cen), cen.shape[0], _p(x), _p(y), _p(z), len(x),
                           out.ctypes.data_as(ctypes.POINTER(ctypes.c_long)))
    return out


def select_patch(patch, centers, x, y, z=None):
    """SelectPatch (src/KMeans.cpp:944-1011) restated."""
    cen = np.ascontiguousarray(centers, dtype=float)
    x = np.ascontiguousarray(x, dtype=float)
    y = np.ascontiguousarray(y, dtype=float)
    z = None if z is None else np.ascontiguousarray(z, dtype=float)
    out = np.empty(len(x), dtype=np.int64)
    lib().orc_select_patch(int(patch), _p(cen), cen.shape[0], _p(x), _p(y), _p(z), len(x),
                           out.ctypes.data_as(ctypes.POINTER(ctypes.c_long)))
    return out
