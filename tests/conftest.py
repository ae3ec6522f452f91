"""Shared test set-up: the `gpu` marker, builds of the library and the
oracle, and golden-fixture helpers."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Builds libwalkray_gpu.so and the oracle once per session."""
    from walkray_gb300 import build

    build.build_lib()
    build.build_oracle()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    from walkray_gb300.api import Context

    c = Context()
    yield c
    c.close()
