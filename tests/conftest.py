import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cu-reconstruction_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def oracle():
    import oracle as o
    o.ensure_built()
    return o


@pytest.fixture(scope="session")
def engine_lib():
    """Builds (if stale) and loads the engine library; no GPU needed."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("gbt_engine_build", os.path.join(PKG, "build.py"))
    engine_build = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(engine_build)
    engine_build.build()
    from cuphoto import _lib
    return _lib


@pytest.fixture(scope="session")
def gpu(engine_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need CUDA; the engine has no CPU path")
    torch.cuda.init()
    return torch
