import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT / "csmv-gpu-stm_gb300", ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (run with -m gpu)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Make sure the library and the checker exist (the harness calls build() first too)."""
    from csmv_gb300 import build as b

    import oracle

    if not b.LIB.exists():
        b.build()
    oracle.build()
    yield
