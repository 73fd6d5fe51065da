"""Shared fixtures.  Tests marked `gpu` need a CUDA device (run with
`-m gpu`); everything else runs on the CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_fixtures.npz")
# the reference's own answers on the two benchmarked plain-method workloads
# (tests/golden/make_golden_configs.py)
GOLDEN_CONFIGS = os.path.join(ROOT, "tests", "golden", "reference_configs.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def golden_configs():
    return np.load(GOLDEN_CONFIGS)


@pytest.fixture(scope="session")
def golden_cases(golden):
    return [str(c) for c in golden["index/cases"]]


@pytest.fixture(scope="session")
def cp():
    """The library, built and loaded; fails loudly without a GPU."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    from cpvs_gb300 import build
    build.build()
    import cpvs_gb300
    cpvs_gb300.load_library()
    return cpvs_gb300
