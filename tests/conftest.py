import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tensorcrossinterpolation.jl_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs libtci_gpu.so kernels)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "reference_known_answers.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.lib()
    return O


@pytest.fixture(scope="session")
def T():
    """The product package with its CUDA library loaded (GPU tests only)."""
    import tci_gb300

    tci_gb300.load_library()
    return tci_gb300
