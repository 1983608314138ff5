import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import oracle_io  # noqa: E402

# the reference checkout where present (None on machines without it)
REFERENCE = oracle_io.reference_dir()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300)")


@pytest.fixture(scope="session")
def oracle_built():
    oracle_io.build(REFERENCE)
    return oracle_io


@pytest.fixture(scope="session")
def engine_lib():
    from mytrim_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def gpu_engine(engine_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test without a CUDA device")
    from mytrim_gb300 import Engine
    e = Engine(precision="fp64")
    yield e
    e.close()
