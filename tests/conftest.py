import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) device")


@pytest.fixture(scope="session")
def covlib():
    """libcovgpu.so, built in-tree when missing (nvcc cross-compiles here)."""
    from coldcase_gb300 import _build, lib
    if not os.path.exists(_build.lib_path()):
        _build.build()
    return lib.load()


@pytest.fixture(scope="session")
def golden():
    import json
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    with open(os.path.join(here, "engine_runs.json")) as f:
        runs = json.load(f)
    with open(os.path.join(here, "verify_cases.json")) as f:
        cases = json.load(f)
    return runs, cases


@pytest.fixture(scope="session")
def sym_golden():
    """The reference quotient search's runs (tests/golden/sym_runs.json)."""
    import json
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    with open(os.path.join(here, "sym_runs.json")) as f:
        return json.load(f)
