import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def lib_built():
    from transportoptimiser_gb300 import build
    build.build()
    return build.LIB


@pytest.fixture(scope="session")
def ctx(lib_built):
    from transportoptimiser_gb300._capi import Context
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    d = ROOT / "tests" / "golden"
    return {p.stem: dict(np.load(p)) for p in d.glob("*.npz")}
