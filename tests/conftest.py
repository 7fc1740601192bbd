"""Shared fixtures. GPU tests carry @pytest.mark.gpu; the rest run on CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


_cache = {}


def detector(preset):
    from acts_gb300 import generate

    if ("det", preset) not in _cache:
        _cache[("det", preset)] = generate.Detector(preset)
    return _cache[("det", preset)]


def batch(preset, n, seed=11):
    from acts_gb300 import generate

    key = ("batch", preset, n, seed)
    if key not in _cache:
        _cache[key] = generate.generate(detector(preset), n, seed=seed)
    return _cache[key]


@pytest.fixture(scope="session")
def fitter_factory():
    """CudaKalman per preset, created lazily (GPU tests only)."""
    from acts_gb300.fitter import CudaKalman

    made = {}

    def get(preset):
        if preset not in made:
            made[preset] = CudaKalman.for_detector(detector(preset))
        return made[preset]

    yield get
    for f in made.values():
        f.close()
