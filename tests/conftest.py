import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def _native_build():
    """Builds the native libraries once per session (no-op when up to date)."""
    from oracle import build as oracle_build
    from visionaray_gb300 import build
    build.build()
    oracle_build.build()


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def golden():
    import json
    import numpy as np
    here = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(here, "golden.json")) as f:
        meta = json.load(f)
    samples = dict(np.load(os.path.join(here, "golden_samples.npz")))
    return meta, samples
