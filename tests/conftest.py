import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    return pyoracle.Oracle()


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name)) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session", params=["plummer_s4.npz", "nfw_s16.npz"])
def golden(request):
    return load_golden(request.param)


@pytest.fixture(scope="session")
def gpu_ctx():
    from asmooth_gb300 import build as B
    from asmooth_gb300 import api

    B.build()
    ctx = api.Context(0)
    yield ctx
    ctx.close()
