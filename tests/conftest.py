import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the sm_103a kernels")


def pytest_runtest_setup(item):
    if "gpu" in item.keywords:
        import torch

        if not torch.cuda.is_available():
            pytest.fail("this test needs a CUDA device (the synthesis path has no CPU fallback)")


@pytest.fixture(scope="session")
def golden():
    return GOLDEN
