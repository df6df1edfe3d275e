import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def product_lib():
    from minirender_gb300 import build, capi
    build.build()
    return capi.lib()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O
    O.build(with_ref=False)
    return O.lib()


@pytest.fixture(scope="session")
def ref_lib():
    from oracle import oracle as O
    L = O.ref_lib()
    if L is None:
        pytest.skip("reference sources not present on this machine")
    return L


@pytest.fixture(scope="session")
def gpu_ctx(product_lib):
    from minirender_gb300 import capi
    ctx = capi.Context(0)
    yield ctx
    ctx.close()
