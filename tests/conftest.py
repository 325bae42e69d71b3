import os
import sys
import pathlib

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmfx.so")


@pytest.fixture(scope="session")
def mfxlib():
    from monofonic_gb300 import build, mfx
    build.build()
    return mfx


@pytest.fixture(scope="session")
def engine(mfxlib):
    import torch  # noqa: F401  (only to report a clear skip reason)
    eng = mfxlib.Engine(0)
    yield eng
    eng.close()


@pytest.fixture(scope="session")
def oracle():
    from oracle import lpt
    lpt.build_lib()
    return lpt
