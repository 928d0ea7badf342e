import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda():
    if not has_gpu():
        pytest.skip("no CUDA device")
    import torch
    import later_gb300
    later_gb300.lib()
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def ref(cuda):
    """The reference LATER on the GPU (oracle/_ref: its kernels + restated host code), or skip."""
    from oracle import build_ref
    if not build_ref.available():
        build_ref.build()
    r = build_ref.load()
    if r is None:
        pytest.skip("oracle/_ref (the reference's kernels and harness) is not built")
    return r
