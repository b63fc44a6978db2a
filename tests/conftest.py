import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


class Golden:
    """Access to tests/golden/golden.npz as golden[case][key]."""

    def __init__(self, path):
        self._z = np.load(path, allow_pickle=False)
        self.cases = sorted({k.split("/")[0] for k in self._z.files})

    def __getitem__(self, case):
        pre = case + "/"
        return {k[len(pre):]: self._z[k] for k in self._z.files if k.startswith(pre)}


@pytest.fixture(scope="session")
def golden():
    return Golden(GOLDEN)


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build()
    return oracle


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def vg():
    """The vir_gb300 package with its CUDA library loaded (GPU tests only)."""
    if not gpu_available():
        pytest.skip("no CUDA device")
    import vir_gb300
    vir_gb300.load()
    return vir_gb300
