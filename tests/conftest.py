import json
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PACKAGE = ROOT / "heronian-square-search_gb300"
GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(PACKAGE))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: long CPU runs, enabled with HSS_SLOW=1")


def pytest_collection_modifyitems(config, items):
    if os.environ.get("HSS_SLOW") == "1":
        return
    skip = pytest.mark.skip(reason="slow; set HSS_SLOW=1")
    for item in items:
        if "slow" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def built():
    """Builds libhss.so, the CLI and the oracle in-tree (make is incremental)."""
    sys.path.insert(0, str(ROOT))
    import __graft_entry__

    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def golden_runs():
    return json.loads((GOLDEN / "reference_runs.json").read_text())["runs"]


@pytest.fixture(scope="session")
def published():
    return json.loads((GOLDEN / "published.json").read_text())
