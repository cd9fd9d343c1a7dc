import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the oracle (C restatement, and the reference's own CPU sources
    when the reference checkout is present) and the CUDA library once."""
    from oracle import oracle as O
    O.build()
    from libfalcon_dsp_gb300 import build as B
    B.build()
    yield
