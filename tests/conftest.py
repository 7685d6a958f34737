import os
import sys
import tempfile

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN_DIR = os.path.join(REPO, "tests", "golden")
GOLDEN_CASES = ["l2_int_d32", "cos_d24", "l2_d30_lsq5", "l2_small_heap", "pq_l2_int_d32", "pq_cos_d24",
                "ip2cos_d23"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    """Returns (npz, index_dir) with the reference-built index written to a temp dir."""
    from puck_gb300 import index_io
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    d = tempfile.mkdtemp(prefix=f"puck_golden_{name}_")
    index_io.materialize_npz_index(z, d)
    return z, d


@pytest.fixture(scope="session", params=GOLDEN_CASES)
def golden(request):
    return (request.param,) + load_golden(request.param)


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
