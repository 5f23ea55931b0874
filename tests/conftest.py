import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gala-mg_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def ffi():
    import gala_ffi
    if not os.path.exists(gala_ffi.LIB_PATH):
        import build as gbuild
        gbuild.build()
    gala_ffi.load()
    return gala_ffi


@pytest.fixture(scope="session")
def oracle():
    from oracle_ffi import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def mlp_oracle():
    """FP64 CPU restatement of the move-proposal network (oracle/mlp_oracle.py)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("mlp_oracle", os.path.join(ROOT, "oracle", "mlp_oracle.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def golden():
    return GOLDEN
