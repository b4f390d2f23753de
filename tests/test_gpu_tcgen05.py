"""The tcgen05 building blocks (shared-memory descriptors, the TF32 instruction
descriptor, TMEM accumulators) on one 128-row tile against numpy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,k", [(16, 8), (48, 32), (64, 64)])
def test_tcgen05_integer_gemm_exact(gpu_lib, n, k):
    rng = np.random.default_rng(n + k)
    a = rng.integers(-8, 9, (128, k)).astype(np.float32)   # exact in TF32, exact sums
    b = rng.integers(-8, 9, (n, k)).astype(np.float32)
    c = gpu_lib.tcgen05_selftest(a, b)
    assert np.array_equal(c, a @ b.T)


def test_tcgen05_tf32_accuracy(gpu_lib):
    rng = np.random.default_rng(3)
    a = rng.normal(size=(128, 64)).astype(np.float32)
    b = rng.normal(size=(48, 64)).astype(np.float32)
    c = gpu_lib.tcgen05_selftest(a, b)
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    assert np.abs(c - ref).max() <= 2e-3 * np.abs(ref).max()
