import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT / "h-blast_gb300", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Build the CUDA library and the oracle once per session (no GPU needed;
    nvcc cross-compiles), so that every test finds them in a fresh checkout."""
    import __graft_entry__ as g
    g.build()
    return True
