"""CPU restatement of TreeCorr's jackknife covariance for 2-point results -- test
infrastructure only.

Follows treecorr/corr2base.py: JackknifePairIterator (1787-1817) for the pair weights,
_sum (1333-1352) and _finalize (1274-1294) for a row, getStat (GG: xip then xim; KK: xi),
and _cov_jackknife (2432-2445) for C = (1 - 1/npatch) sum (v - mean)(v - mean)^T.
results: [npair, 8, nbins] = weight, meanr, meanlogr, xi0..xi3, npairs.
"""
import numpy as np


def pair_weight(l, i, j, npatch, cpw):
    if cpw == "simple":
        return 1.0 if (i != l and j != l) else 0.0
    if i == l and j == l:
        return 0.0
    if i == l or j == l:
        if cpw == "mean":
            return 0.5
        return 1 - npatch / (2 + 2 ** 0.5 * (npatch - 1))     # match
    return 1.0


def design_matrix(results, pairs, npatch, gg=True, cpw="simple"):
    nb = results.shape[2]
    rows = []
    for l in range(npatch):
        w = np.zeros(nb)
        xi = np.zeros((4, nb))
        for (i, j), r in zip(pairs, results):
            pw = pair_weight(l, i, j, npatch, cpw)
            if pw == 0:
                continue
            w += pw * r[0]
            xi += pw * r[3:7]
        mask = w != 0
        xi[:, mask] /= w[mask]
        xi[:, ~mask] = 0.
        rows.append(np.concatenate([xi[0], xi[2]]) if gg else xi[0].copy())
    return np.array(rows)


def cov_jackknife(v):
    n = v.shape[0]
    d = v - v.mean(axis=0)
    return (1. - 1. / n) * d.conj().T.dot(d)
