import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA library through its C ABI)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(ROOT, "tests", "golden", "reference_values.json")) as f:
        return json.load(f)


def fv_cell_average_1d(ncell, func, order):
    """FiniteVolume interpolation of the reference (spaces/basis/finite-volume.hh:244-252):
    element integral with a quadrature of the function's order, divided by the volume."""
    m = order // 2 + 1
    x, w = np.polynomial.legendre.leggauss(m)
    x, w = (x + 1) / 2, w / 2
    h = 1.0 / ncell
    left = np.arange(ncell) * h
    return sum(wq * func(left + xq * h) for xq, wq in zip(x, w))


def import_gdt():
    import importlib

    return importlib.import_module("dune-gdt_gb300")


@pytest.fixture(scope="session")
def gdt():
    """The GB300 package; GPU tests need the CUDA library built in-tree (no fallback)."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    mod = import_gdt()
    mod._capi.load(build_if_missing=True)
    return mod


def csr_equal_pattern(gpu_csr, orc):
    rp, col, _ = gpu_csr
    return (np.array_equal(rp.cpu().numpy().astype(np.int64), orc.row_ptr)
            and np.array_equal(col.cpu().numpy(), orc.col))


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
