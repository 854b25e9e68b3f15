import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300)")
    config.addinivalue_line("markers", "slow: full-size configuration (minutes)")


@pytest.fixture(scope="session", autouse=True)
def _built_library():
    """Compile libkcore.so and the oracle once per session (incremental)."""
    from pico_gb300 import build as pb
    pb.build()
    import oracle
    oracle.build()
    yield


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(TESTS, "golden", "reference_loaders.json")) as f:
        return json.load(f)


@pytest.fixture
def mtx_file(tmp_path):
    def write(text, name="g.mtx"):
        p = tmp_path / name
        p.write_text(text)
        return str(p)
    return write
