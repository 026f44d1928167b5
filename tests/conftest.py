import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def asv():
    import anisotropic_supervoxel_gb300 as a
    a.load()
    return a


def small_clip(asv, W=64, H=48, D=12, seed=7, n_ellipses=6, noise=5.0, jitter=0.0, drift=0.0):
    return asv.synth_clip(W, H, D, n_ellipses=n_ellipses, noise_sigma=noise, vmax=3.0,
                          jitter=jitter, drift_amp=drift, drift_period=20.0, seed=seed)


@pytest.fixture
def clip_small(asv):
    return small_clip(asv)


def mismatch(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return int((a != b).sum())
