import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.lib()
    return O


def _have_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def hg():
    """The CUDA library, built if needed.  GPU tests only."""
    if not _have_gpu():
        pytest.fail("GPU test collected without a GPU")
    from hypergeometrica_gb300 import build as B

    B.build()
    import hypergeometrica_gb300 as H

    H.init()
    return H


def h2i(v):
    return [int(x, 16) for x in v]
