"""Test configuration: import paths, the `gpu` marker and shared helpers.

`-m "not gpu"` runs the oracle against the reference's golden vectors, the host logic
and the library's export table (no GPU).  `-m gpu` runs the parity tests proper: the
CUDA library through its C ABI against the oracle.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "splinegrids.jl_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU; runs the CUDA library")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def sg():
    """The package with its CUDA library built; fails (does not skip) without a GPU."""
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA; the library has no CPU path"
    sys.path.insert(0, os.path.join(ROOT, "splinegrids.jl_gb300"))
    import build as sg_build
    sg_build.build()
    import splinegrids
    splinegrids.load_library()
    return splinegrids


def normwise_rel(a, ref) -> float:
    """max|a - ref| / max|ref| (the error measure of the parity bar)."""
    a = np.asarray(a, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = np.abs(ref).max() if ref.size else 1.0
    return float(np.abs(a - ref).max() / (den if den > 0 else 1.0)) if ref.size else 0.0
