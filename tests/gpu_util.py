"""Shared helpers of the GPU tests."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


# Tolerances.  The plain FP32 path reproduces the reference's float
# operations in order, so the filters are compared bit for bit (== , which
# treats -0.0 and +0.0 as equal).  The slope estimate goes through
# conjugate-gradient iterations whose rounding the reference's own FP32
# arithmetic already amplifies to ~1e-4 on noisy data; it is held to the
# stated bar of 1e-4 relative L2.
DIP_TOL = 1e-4
