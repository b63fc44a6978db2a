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


def voxel_sphere(n, d, sphere, sub=4, mu=1.0):
    """(n, n, n) volume of cubic voxels d (centred grid) holding a sphere
    (x0, y0, z0, r) of attenuation mu, each voxel the fraction of its sub^3
    sample points inside."""
    ax = d * (np.arange(n) + 0.5 - n / 2)
    off = ((np.arange(sub) + 0.5) / sub - 0.5) * d
    x0, y0, z0, r = (float(v) for v in sphere)
    vol = np.zeros((n, n, n))
    for a in off:
        dx2 = (ax + a - x0)[:, None, None] ** 2
        for b in off:
            dy2 = (ax + b - y0)[None, :, None] ** 2
            for c in off:
                vol += (dx2 + dy2 + (ax + c - z0)[None, None, :] ** 2) <= r * r
    return vol * (mu / sub ** 3)


@pytest.fixture(scope="session")
def sphere_vol():
    return voxel_sphere
