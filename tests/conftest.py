import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


@pytest.fixture(scope="session")
def gpu_context():
    """The product's CUDA context on device 0 (GPU tests only; fails loudly without one)."""
    from gartus_gb300 import build as gbuild
    from gartus_gb300.raytracing import Context
    gbuild.build()
    return Context.default()
