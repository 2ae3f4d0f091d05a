import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native_lib():
    import pamo_gb300._build as b

    b.build()
    import pamo_gb300._native as n

    return n.load()


@pytest.fixture(scope="session")
def torch_ext():
    """The extension module pamo_gb300._C (built with the library)."""
    import pamo_gb300._build as b

    b.build()
    import torch  # noqa: F401  (loads the torch libraries the module links)

    import pamo_gb300._C as C

    return C
