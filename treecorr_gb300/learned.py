"""The learned opening criterion: training data from the traversal, training on the GPU,
and its use in GGCorr / KKCorr / NNCorr processing (no reference counterpart).

The bin_slop rule of the reference (include/BinType.h:93-151) splits every cell pair whose
size is large against b * r.  Among those, pairs far from a bin edge can be accepted at a
small cost: almost all of their point pairs fall in the same bin.  The network predicts
log10 of the weight fraction that would fall in another bin (the "leak") from five
features, and the traversal accepts a candidate pair when the prediction is below a
threshold.  Training pairs come from a traversal with the plain rule (sampled candidates,
each recounted point by point on the GPU); training uses the library's own forward /
backward / Adam kernels.
"""
import numpy as np

from . import _treecorr as T

NIN, NH = 5, 64


def init_params(seed=0):
    """He-uniform initial parameters (FP32)."""
    rng = np.random.default_rng(seed)
    def he(fan_in, shape):
        lim = np.sqrt(6.0 / fan_in)
        return rng.uniform(-lim, lim, size=shape)
    parts = [he(NIN, (NH, NIN)).ravel(), np.zeros(NH), he(NH, (NH, NH)).ravel(), np.zeros(NH),
             he(NH, NH) * 0.1, np.array([-3.0])]
    p = np.concatenate(parts).astype(np.float32)
    assert len(p) == T.mlp_nparam()
    return p


def collect(corr, field, metric, sample_mod=16, max_samples=1 << 20, max_point_pairs=1 << 16):
    """Training pairs from one processAuto with the bin_slop rule; drops unlabelled ones."""
    x, y = corr.learnCollect(field, metric, sample_mod, max_samples, max_point_pairs)
    ok = np.isfinite(y)
    return x[ok], y[ok]


def train(x, y, steps=3000, batch=4096, lr=2e-3, seed=0, params=None):
    """Train on (features, log10 leak targets); returns (params, loss per step)."""
    p0 = init_params(seed) if params is None else params
    return T.mlp_train(p0, x, y, steps, batch=batch, lr=lr, seed=seed)
