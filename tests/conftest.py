import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests proper")


@pytest.fixture(scope="session")
def built():
    """libsplgpu.so and the oracle port, compiled in-tree (no-op when fresh)."""
    from oracle import oracle
    from splotch_gb300 import build as b

    b.build()
    oracle.build_port()
    return True


@pytest.fixture(scope="session")
def port(built):
    from oracle.oracle import Port

    return Port()


@pytest.fixture(scope="session")
def renderer(built):
    import splotch_gb300 as sg

    r = sg.Renderer(0)
    yield r
    r.close()
