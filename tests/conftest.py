import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libnsg.so")


@pytest.fixture(scope="session")
def nsg_ctx():
    """A device context on cuda:0 (builds libnsg.so if needed)."""
    import networksolvers_gb300.build as nb
    from networksolvers_gb300 import _native
    nb.build()
    ctx = _native.Context(0)
    _native.set_default_context(ctx)
    yield ctx
    ctx.synchronize()
