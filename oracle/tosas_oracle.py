"""Oracle (test infrastructure only): a numpy restatement of what TreeCorr's Python layer
does with a GGG LogMultipole result to turn it into LogSAS binning -- the multipole
normalisation of the mean distances (Corr3._finalize, treecorr/corr3base.py:2312-2396) and
toSAS (treecorr/corr3base.py:2553-2676) with the x-to-centroid projection phases
(_x_to_natural_phases, treecorr/corr3base.py:2489-2552).  The tests feed it the raw outputs
of the GGGCorr process call -- the reference module's, logged by
tests/golden/make_api_trace.py, and this module's, replayed on the GPU -- and compare with
the LogSAS result TreeCorr's own Python computed.  Only tests/ import this module.
"""
import numpy as np


def ggg_multipole_to_sas(outs, nbins, max_n, min_sep, bin_size, phi):
    """outs: the 19 output arrays of GGGCorr after its process calls (zeta0..7, meand1,
    meanlogd1, meand2, meanlogd2, meand3, meanlogd3, meanu, meanv, weight, weight_im, ntri;
    raw sums, as the native module leaves them), for a flat catalog without units.  phi: the
    LogSAS phi grid [nbins, nbins, nphi] in radians.  Returns (weight, [gam0, gam1, gam2,
    gam3]) of the LogSAS correlation."""
    nn = 2 * max_n + 1
    shp = (nbins, nbins, nn)
    z = [np.asarray(a, dtype=float).reshape(shp) for a in outs[:8]]
    meand2 = np.asarray(outs[10], dtype=float).reshape(shp)
    meand3 = np.asarray(outs[12], dtype=float).reshape(shp)
    weightr = np.asarray(outs[16], dtype=float).reshape(shp)
    weighti = np.asarray(outs[17], dtype=float).reshape(shp)
    # Corr3._finalize for LogMultipole: the mean distances over the weight (the native module
    # sets them at n = 0, index max_n, where the weight is the plain sum of w w w), the
    # nominal distances (log-bin centres) where there are no triangles, then that plane
    # broadcast over n; zeta stays raw.
    w0 = weightr[:, :, max_n]
    rnom = np.exp(np.log(min_sep) + (np.arange(nbins) + 0.5) * bin_size)
    d2nom = np.broadcast_to(rnom[:, None], (nbins, nbins))
    d3nom = np.broadcast_to(rnom[None, :], (nbins, nbins))
    m0 = w0 != 0
    d2 = np.where(m0, meand2[:, :, max_n] / np.where(m0, w0, 1.), d2nom)
    d3 = np.where(m0, meand3[:, :, max_n] / np.where(m0, w0, 1.), d3nom)
    weight = weightr + 1j * weighti
    gams = [z[2 * k] + 1j * z[2 * k + 1] for k in range(4)]
    # toSAS: N(d2, d3, phi) = 1/2pi sum_n N_n(d2, d3) exp(i n phi) over the phi bins.
    phi1d = np.asarray(phi)[0, 0, :]
    dphi = phi1d[1] - phi1d[0] if len(phi1d) > 1 else np.pi
    n1d = np.arange(-max_n, max_n + 1)
    expiphi = np.exp(1j * n1d[:, None] * phi1d)
    wr = np.real(weight.dot(expiphi)) / (2 * np.pi) * dphi
    zs = [g.dot(expiphi) / (2 * np.pi) * dphi for g in gams]
    m = wr != 0
    for zz in zs:
        zz[m] /= wr[m]
    # The x projection of the multipole algorithm to the centroid projection.
    s = np.repeat(d2[:, :, None], len(phi1d), axis=2)
    t = np.repeat(d3[:, :, None], len(phi1d), axis=2) * np.exp(1j * np.asarray(phi))
    u = (1 + t / np.abs(t)) / 2
    q1 = (s + t) / 3.
    q2 = q1 - t
    q3 = q1 - s
    p1 = (u * np.conj(q1)) ** 2
    p2 = (t * np.conj(q2)) ** 2
    p3 = (s * np.conj(q3)) ** 2
    p1 /= np.abs(p1)
    p2 /= np.abs(p2)
    p3 /= np.abs(p3)
    phases = [p1 * p2 * p3, np.conj(p1) * p2 * p3, p1 * np.conj(p2) * p3,
              p1 * p2 * np.conj(p3)]
    return wr, [zz * p for zz, p in zip(zs, phases)]
