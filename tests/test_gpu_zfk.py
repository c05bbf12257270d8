"""FK dip filter on the GPU (pwd_fkdip through fkdip) against the
reference's own outputs (golden_fk.npz) and the oracle: 1e-6 relative L2 for
float32 input (complex64 forward FFTs on both sides, rounded differently),
1e-12 for float64.  The file name sorts after the other GPU tests of the
path."""
import json
import os

import numpy as np
import pytest

from gpu_util import need_gpu, rel_l2

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_fk.npz")
TOL32, TOL64 = 1e-6, 1e-12


@pytest.fixture(scope="module")
def ps():
    need_gpu()
    import pyseistr_gb300

    return pyseistr_gb300


def test_fkdip_matches_reference(ps):
    z = np.load(GOLDEN)
    for m in json.loads(bytes(z["meta"]).decode()):
        k = m["k"]
        d, want = z[f"in_{k}"], z[f"out_{k}"]
        got = ps.fkdip(d, m["w"])
        assert got.dtype == np.float64 and got.shape == want.shape
        assert rel_l2(got, want) <= (TOL64 if d.dtype == np.float64 else TOL32), k


CASES = [
    # n1, n2, w, dtype, seed
    (1000, 960, 0.05, np.float32, 11),   # a DAS window's shape (the demo's w)
    (300, 97, 0.01, np.float32, 12),
    (100, 30, 0.05, np.float64, 13),
    (1, 5, 0.2, np.float32, 14),
    (7, 1, 0.3, np.float32, 15),
    (257, 129, -0.03, np.float32, 16),
]


@pytest.mark.parametrize("case", CASES, ids=[f"fk-{c[0]}x{c[1]}-w{c[2]}-{np.dtype(c[3]).name}"
                                             for c in CASES])
def test_fkdip_matches_oracle(ps, case):
    from oracle import fk_oracle as F

    n1, n2, w, dt, seed = case
    d = np.random.default_rng(seed).standard_normal((n1, n2)).astype(dt)
    got = ps.fkdip(d, w)
    assert got.dtype == np.float64 and got.shape == (n1, n2)
    assert rel_l2(got, F.fkdip(d, w)) <= (TOL64 if dt == np.float64 else TOL32)


def test_fkdip_device_tensors_and_linearity(ps):
    """A CUDA tensor gives the same values as NumPy, repeated calls the same
    bits, and the filter is linear (to the complex64 FFTs' rounding)."""
    import torch

    d = np.random.default_rng(21).standard_normal((200, 64)).astype(np.float32)
    a = ps.fkdip(d, 0.05)
    b = ps.fkdip(torch.from_numpy(d).cuda(), 0.05)
    assert isinstance(b, torch.Tensor) and b.is_cuda and b.dtype == torch.float64
    assert np.array_equal(b.cpu().numpy(), a)
    assert np.array_equal(ps.fkdip(d, 0.05), a)
    e = np.random.default_rng(22).standard_normal((200, 64)).astype(np.float32)
    both = ps.fkdip((2 * d - 3 * e).astype(np.float32), 0.05)
    assert rel_l2(both, 2 * a - 3 * ps.fkdip(e, 0.05)) <= 1e-5


def test_fkdip_shared_memory_transforms_equal_the_passes(ps, monkeypatch):
    """The transforms run in shared memory (one launch each) give the bits
    of the pass-by-pass kernels; a section wide enough that its complex128
    space transforms (nk = 8192) exceed shared memory mixes both forms."""
    from oracle import fk_oracle as F

    for shape in ((300, 97), (64, 5000)):
        d = np.random.default_rng(31).standard_normal(shape).astype(np.float32)
        a = ps.fkdip(d, 0.05)
        monkeypatch.setenv("PWD_FK_SMEM", "0")
        b = ps.fkdip(d, 0.05)
        monkeypatch.delenv("PWD_FK_SMEM")
        assert np.array_equal(a, b)
        assert rel_l2(a, F.fkdip(d, 0.05)) <= TOL32


def test_fkdip_zero_width_raises_like_the_reference(ps):
    with pytest.raises(ZeroDivisionError):
        ps.fkdip(np.zeros((8, 8), np.float32), 0.0)
