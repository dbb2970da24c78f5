import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line(
        'markers', 'gpu: needs a GB300 (sm_103a) GPU and the built library')


def gpu_available():
    try:
        import torch
        if not torch.cuda.is_available():
            return False
        return torch.cuda.get_device_capability(0) == (10, 3)
    except Exception:  # noqa: BLE001
        return False


@pytest.fixture(scope='session')
def golden():
    import numpy as np
    return np.load(os.path.join(REPO, 'tests', 'golden',
                                'reference_vectors.npz'))
