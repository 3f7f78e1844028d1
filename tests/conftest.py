import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")
    config.addinivalue_line("markers", "slow: full-size workloads")


def load_golden(name):
    """(ids uint32, dists float32) of a committed reference output, plus its inputs."""
    from tests.golden.make_golden import case, inputs
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    x, q, k, metric, extra = inputs(case(name))
    return z["ids"], z["dists"], x, q, k, metric, extra


@pytest.fixture(scope="session")
def gpu_ready():
    """Builds the extension if needed; skips cleanly only when there is no GPU."""
    import vecsearch_gb300.build as b
    b.build()
    import vecsearch_gb300 as vsg
    if not vsg.cuda_available():
        pytest.skip("no CUDA device")
    return vsg
