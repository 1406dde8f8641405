import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "mossco-code_gb300"), os.path.join(ROOT, "oracle"),
          ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if gpu_available():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


def relerr(x, ref, floor_frac=1e-4):
    """Max relative error per tracer: |x-ref| / (|ref| + floor), the floor
    being floor_frac times the tracer's largest |ref| over the grid (deep O2
    and NO3 fall to ~0, where a pure relative error is meaningless)."""
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    out = []
    for n in range(ref.shape[0]):
        r = ref[n]
        floor = floor_frac * max(np.max(np.abs(r)), 1e-300)
        out.append(float(np.max(np.abs(x[n] - r) / (np.abs(r) + floor))))
    return np.array(out)
