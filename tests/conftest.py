import json
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden" / "golden.json"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libvoss.so")
    config.addinivalue_line("markers", "slow: long-running parity case")


@pytest.fixture(scope="session")
def golden():
    return json.loads(GOLDEN.read_text())


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


def build_library():
    """Build libvoss.so (voss_gb300/build.py loaded by path, since importing
    the package needs the library)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("voss_gb300_build", ROOT / "voss_gb300" / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


@pytest.fixture(scope="session")
def vg():
    """The GB300 library; builds it if needed and requires a GPU."""
    build_library()
    import voss_gb300
    return voss_gb300
