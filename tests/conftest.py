import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden" / "ref_cpu_golden.npz"

# The drop-in libraries append to gpu_stats.txt in the working directory, as the
# reference does; keep the test tree clean.
os.environ.setdefault("LSGB_NO_STATS", "1")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def native_libs():
    """Build the native libraries if needed (nvcc cross-compiles without a GPU)."""
    from gpu_lomb_scargle_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def cuda_ok():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return True
