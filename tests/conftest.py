import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")
    config.addinivalue_line("markers", "slow: full-size configuration (minutes)")


@pytest.fixture(scope="session")
def built():
    """Builds (if stale) the CUDA library and the oracle."""
    from metada_gb300 import build

    build.build_library()
    build.build_oracle()
    return True


@pytest.fixture(scope="session")
def dev(built):
    import torch

    # GPU tests must run on a GPU: no silent skip, no fallback.
    assert torch.cuda.is_available(), "GPU test run without a CUDA device"
    return torch.device("cuda:0")


def rel_err(a, b):
    import numpy as np

    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (scale if scale > 0 else 1.0))
