import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "dcs_golden.npz")
ELASTIC_GOLDEN = os.path.join(ROOT, "tests", "golden", "elastic_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Builds the CUDA library and the CPU oracle in place if they are missing or stale."""
    from noa_gb300 import build
    return build.build_all(ref=False)


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def elastic_golden():
    with np.load(ELASTIC_GOLDEN) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def cuda_device(built):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
