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


def means_agree(a, b, rel):
    """The image means of two stacks of independent renders (render axis
    first) agree: within `rel` of b's mean, or within 4 standard errors of
    the difference where the renders are noisier than that."""
    import numpy as np

    ma = a.reshape(len(a), -1).mean(1)
    mb = b.reshape(len(b), -1).mean(1)
    se = np.sqrt(ma.var(ddof=1) / len(ma) + mb.var(ddof=1) / len(mb))
    return abs(ma.mean() - mb.mean()) <= max(rel * abs(mb.mean()), 4 * se)


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
