import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def _build_all():
    # the library and the oracle are in-tree build products (git-ignored): build them when
    # missing or stale, so a fresh checkout tests what its sources say
    from feellgood_gb300 import build as fb
    from oracle import build as ob
    fb.build()
    ob.build()


def pytest_configure(config):
    _build_all()
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built fggpu library")


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN
