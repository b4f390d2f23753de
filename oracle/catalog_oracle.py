"""Oracle (test infrastructure only): a numpy restatement of the column work of TreeCorr's
Catalog._finish_input (treecorr/catalog.py:1343-1487) -- flag -> weight, the NaN checks,
the wpos == 0 rule, sumw and the removal of zero-weight rows -- which the GPU's
tc_catalog_finish is checked against.  Pinned to the reference's own Catalog by the
fixtures tests/golden/catalog_*.npz (tests/golden/make_catalog_golden.py).

Only tests/ import this module.
"""
import numpy as np

# The order of the reference's checkForNaN calls (treecorr/catalog.py:1407-1425); w and wpos
# come last.
NAN_ORDER = ("x", "y", "z", "ra", "dec", "r", "k", "z1", "z2", "v1", "v2", "g1", "g2",
             "t1", "t2", "q1", "q2")


def finish_input(cols, w=None, wpos=None, flag=None, ignore_flag=None, ok_flag=0,
                 keep_zero_weight=False):
    """cols: name -> float64 array (positions and values, names from NAN_ORDER).  Returns
    (cols, w, wpos, info) after the reference's steps; info has sumw, nobj, nontrivial_w,
    nan_counts (by name, then "w", "wpos"), wpos_zero, wpos_conflicts."""
    cols = {k: np.array(v, dtype=float) for k, v in cols.items()}
    n = len(next(iter(cols.values())))
    w = None if w is None else np.array(w, dtype=float)
    wpos = None if wpos is None else np.array(wpos, dtype=float)
    # Flag -> weight (catalog.py:1393-1404).
    if flag is not None:
        ignore = ignore_flag if ignore_flag is not None else ~ok_flag
        if w is None:
            w = np.ones(n)
        bad = (np.asarray(flag) & ignore) != 0
        w[bad] = 0
        if wpos is not None:
            wpos[bad] = 0
    # checkForNaN (catalog.py:1406-1425, 1684-1704).
    nan_counts = {}

    def check(col, name):
        nonlocal w
        if col is None:
            return
        idx = np.where(np.isnan(col))[0]
        nan_counts[name] = len(idx)
        if len(idx):
            if w is None:
                w = np.ones(n)
            w[idx] = 0
            col[idx] = 0

    for name in NAN_ORDER:
        if name in cols:
            check(cols[name], name)
    check(w, "w")
    check(wpos, "wpos")
    # wpos == 0 -> w = 0 (catalog.py:1433-1450).
    wpos_zero = wpos_conflicts = 0
    if wpos is not None and np.any(wpos == 0.):
        wpos_zero = int(np.sum(wpos == 0.))
        if w is None:
            w = np.ones(n)
        else:
            wpos_conflicts = int(np.sum(w[wpos == 0.] != 0.))
        w[wpos == 0.] = 0.
    # sumw (catalog.py:1452-1462).
    if w is not None:
        nontrivial = True
        sumw = float(np.sum(w))
        if sumw == 0:
            raise ValueError("Catalog has invalid sumw == 0")
    else:
        nontrivial = False
        sumw = float(n)
        w = np.ones(n)
    # Removal of zero-weight rows (catalog.py:1464-1468, select 1633-1660).
    if nontrivial and not keep_zero_weight:
        use = (wpos if wpos is not None else w) != 0
        if not np.all(use):
            cols = {k: v[use] for k, v in cols.items()}
            w = w[use]
            wpos = wpos[use] if wpos is not None else None
    nobj = int(np.sum(w != 0)) if nontrivial else len(w)
    info = dict(sumw=sumw, nobj=nobj, nontrivial_w=nontrivial, nan_counts=nan_counts,
                wpos_zero=wpos_zero, wpos_conflicts=wpos_conflicts)
    return cols, w, wpos, info


def center_size(x, y, z=None):
    """Catalog._get_center_size (treecorr/catalog.py:1330-1341): the unweighted mean position
    and the largest distance of a point from it."""
    mx, my = np.mean(x), np.mean(y)
    mz = 0
    dsq = (x - mx) ** 2 + (y - my) ** 2
    if z is not None:
        mz = np.mean(z)
        dsq += (z - mz) ** 2
    return mx, my, mz, np.max(dsq) ** 0.5
