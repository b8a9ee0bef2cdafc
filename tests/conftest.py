import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


# GPU test modules in the order they run (under -x a failure stops the rest):
# those that have passed on a GB300 first, the newer ones after them, and the
# allocation-free entry point last.  Other modules keep their place before them.
GPU_ORDER = ("test_gpu_adjoint", "test_gpu_parity", "test_gpu_scale", "test_gpu_ts1", "test_gpu_tuning",
             "test_gpu_tangent", "test_gpu_mechanisms", "test_gpu_reference", "test_gpu_golden", "test_registry",
             "test_solver_kernels", "test_gpu_window_adjoint", "test_gpu_carry", "test_zz_no_alloc")


def _gpu_rank(item):
    name = item.module.__name__.rsplit(".", 1)[-1] if item.module else ""
    return GPU_ORDER.index(name) + 1 if name in GPU_ORDER else 0


def pytest_collection_modifyitems(config, items):
    items.sort(key=_gpu_rank)
    if _cuda_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def built_libs():
    """Build (if stale) and return the mechanism libraries used by GPU tests."""
    from mkpp_gb300 import build

    return build.build(("chapman", "small_strato", "saprc99", "chapman_rodas3", "small_strato_rodas3"))
