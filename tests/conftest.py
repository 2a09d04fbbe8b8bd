import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "dphpc-gpu_mpi_gb300"))
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpulib():
    """Builds libgpumpi.so once per session (on the GPU machine) and returns the gpumpi module."""
    if not has_gpu():
        pytest.skip("no GPU")
    import gpumpi
    gpumpi.build()
    gpumpi.lib()
    return gpumpi


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.build()
    return o
