"""Test configuration: the ``gpu`` marker and shared fixtures.

``-m "not gpu"`` runs everything that needs no GPU (oracle against golden
vectors, host logic, C-ABI exports); ``-m gpu`` runs the parity tests proper,
which call the engine through its C ABI on a GB300.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libhbx.so")
    # the tile-shape autotuner's cache goes to a private file during tests
    import tempfile

    os.environ.setdefault("HBX_AUTOTUNE_CACHE",
                          os.path.join(tempfile.mkdtemp(prefix="hbx_tests_"), "autotune.json"))


@pytest.fixture(scope="session")
def built():
    """Builds the oracle and the engine library once per test session."""
    from oracle import api as oapi
    from hyperblocker_gb300 import build as hbuild

    oapi.build()
    hbuild.build()
    return True


@pytest.fixture(scope="session")
def golden():
    import json

    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        return json.load(f)["cases"]


@pytest.fixture(scope="session")
def ctx(built):
    import hyperblocker_gb300 as hb

    c = hb.Context(0)
    yield c
    c.close()
