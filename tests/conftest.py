"""Shared test setup: repository root on sys.path, the `gpu` marker, and
helpers that build the extension when it is missing."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300)")


def _ensure_built():
    import importlib.util
    spec = importlib.util.spec_from_file_location("_hqs_build", os.path.join(ROOT, "hiqsimulator_gb300", "_build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()


@pytest.fixture(scope="session")
def hqs():
    """The product package (built in place if needed)."""
    _ensure_built()
    import hiqsimulator_gb300
    return hiqsimulator_gb300


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle.lib import load_oracle_lib
    return load_oracle_lib()


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a visible CUDA device")
    return torch
