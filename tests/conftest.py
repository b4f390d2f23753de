import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in-tree if needed; skips nothing -- a GPU test fails loudly
    when the extension is missing."""
    from treecorr_gb300 import build as tb
    tb.build()
    from treecorr_gb300 import _treecorr
    return _treecorr
