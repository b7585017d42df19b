import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "cft-fp256_gb300"))
sys.path.insert(0, str(ROOT / "tests"))
sys.path.insert(1, str(ROOT))              # bench_suites (benchmark and test workloads)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (a GB300); parity tests proper")


def pytest_sessionstart(session):
    """A fresh checkout has no library yet: build it (nvcc cross-compiles
    without a GPU) before any test loads it."""
    import os
    if os.environ.get("CFTG_LIB"):
        return
    from cftgb import build
    if not build.LIB.exists():
        build.build_lib()


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib
    return oracle_lib.Oracle()


@pytest.fixture(scope="session")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a -m gpu test ran without a CUDA device")
    import cftgb
    h = cftgb.open_device("cuda:0")
    yield h
    cftgb.close_device(h)
