import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib():
    from cudatracer_gb300 import _build, _lib

    _build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.build_oracle()
    return oracle


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.fixture(scope="session")
def kat():
    return golden("kat_math.npz")


@pytest.fixture(scope="session")
def c1():
    """The 81,920-triangle sphere scene with the reference's answers."""
    from cudatracer_gb300 import scenes

    g = golden("sphere_c1.npz")
    v, f = scenes.icosphere(int(g["subdivisions"]))
    import hashlib

    assert hashlib.sha256(f.tobytes()).hexdigest() == str(g["indices_sha"])
    return {"g": g, "vertices": g["vertices"], "indices": f}


@pytest.fixture(scope="session")
def gpu_ctx(lib):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cudatracer_gb300 import api

    return api.Context(0)
