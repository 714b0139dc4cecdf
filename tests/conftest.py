import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests", "golden"),
          os.path.join(ROOT, "oracle", "ref_harness")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")

# Parity bar for FP32 results against the reference's kernels and the oracle (relative L2).
REL_L2_TOL = 1e-5


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def rel_l2_group(fields_a, fields_b, c: int) -> float:
    """Error of field component c relative to the norm of its group (E: 0-2, H: 3-5): components
    that are zero by symmetry (Hz of a z-directed source in vacuum) are measured against the
    physical field scale, not against their own rounding noise."""
    g = range(0, 3) if c < 3 else range(3, 6)
    den = np.sqrt(sum(np.linalg.norm(np.asarray(fields_b[q], dtype=np.float64)) ** 2 for q in g))
    num = np.linalg.norm(np.asarray(fields_a[c], dtype=np.float64) - np.asarray(fields_b[c], dtype=np.float64))
    return float(num / den) if den > 0 else float(num)


def bitwise_equal(a, b) -> bool:
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    return a.shape == b.shape and bool(np.array_equal(a.view(np.uint32), b.view(np.uint32)))


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if stale) and load the CUDA library; skip only when no GPU is visible."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fdtd_gb300 import build, solver
    build.build()
    return solver.load_library()
