import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "sampling-graph-mining_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA library)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the library and the oracle once per session (no-op when up to date)."""
    import zgbuild
    zgbuild.build_library()
    zgbuild.build_oracle()
    yield
