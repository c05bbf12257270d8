"""Plane-wave painting on the GPU (pwd_paint2d through pwpaintc / rgt /
cpaint2d) against the reference's own outputs (golden_paint.npz) and the
oracle, bit for bit.  The file name sorts after the other GPU tests of the
path."""
import json
import os

import numpy as np
import pytest

from gpu_util import need_gpu

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_paint.npz")


@pytest.fixture(scope="module")
def ps():
    need_gpu()
    import pyseistr_gb300

    return pyseistr_gb300


def test_pwpaintc_matches_reference(ps):
    z = np.load(GOLDEN)
    for m in json.loads(bytes(z["meta"]).decode()):
        k = m["k"]
        got = ps.pwpaintc(z[f"dip_{k}"], z[f"seed_{k}"], order=m["order"], i0=m["i0"],
                          eps=m["eps"])
        assert got.dtype == np.float32 and got.shape == z[f"dip_{k}"].shape
        assert np.array_equal(got, z[f"out_{k}"]), k


CASES = [
    # n1, n2, order, i0, eps, seed
    (501, 100, 2, 50, 0.1, 11),
    (120, 40, 1, 0, 0.01, 12),
    (97, 33, 3, 32, 0.05, 13),
    (64, 20, 4, 7, 0.01, 14),
    (4, 6, 2, 3, 0.1, 15),
    (50, 1, 2, 0, 0.1, 16),
]


@pytest.mark.parametrize("case", CASES, ids=[f"paint-{c[0]}x{c[1]}-o{c[2]}-i{c[3]}"
                                             for c in CASES])
def test_rgt_matches_oracle(ps, case):
    from oracle import oracle as O

    n1, n2, order, i0, eps, seed = case
    rng = np.random.default_rng(seed)
    dip = (rng.standard_normal((n1, n2)) * 1.5).astype(np.float32)
    got = ps.rgt(dip, o1=0.1, d1=0.004, order=order, i0=i0, eps=eps)
    trace = (np.linspace(0, 0.004 * (n1 - 1), n1) + 0.1).astype(np.float32)
    want = O.paint2d(dip, trace, order=order, i0=i0, eps=eps)
    assert np.array_equal(got, want)


def test_pwpaintc_device_tensors(ps):
    import torch

    rng = np.random.default_rng(21)
    dip = rng.standard_normal((80, 30)).astype(np.float32)
    tr = rng.standard_normal(80).astype(np.float32)
    a = ps.pwpaintc(dip, tr, order=2, i0=10, eps=0.1)
    b = ps.pwpaintc(torch.from_numpy(dip).cuda(), torch.from_numpy(tr).cuda(), order=2, i0=10,
                    eps=0.1)
    assert isinstance(b, torch.Tensor) and b.is_cuda and tuple(b.shape) == (80, 30)
    assert np.array_equal(b.cpu().numpy(), a)


def test_cpaint2d_refuses_bad_arguments(ps):
    dip = np.zeros((16, 4), np.float32)
    with pytest.raises(ValueError):
        ps.cpaint2d(dip, np.zeros(16, np.float32), 16, 4, 2, 4, 0.1, 0)  # i0 = n2
    with pytest.raises(ValueError):
        ps.cpaint2d(dip, np.zeros(16, np.float32), 16, 5, 2, 0, 0.1, 0)  # dimension mismatch
    with pytest.raises(ValueError):
        ps.cpaint2d(dip, np.zeros(8, np.float32), 16, 4, 2, 0, 0.1, 0)   # short seed


def test_pwpaintc_batch_equals_one_call_per_section(ps):
    rng = np.random.default_rng(31)
    dips = [(rng.standard_normal((120, 30)) * 1.2).astype(np.float32) for _ in range(6)]
    seeds = [rng.standard_normal(120).astype(np.float32) for _ in range(6)]
    got = ps.pwpaintc_batch(dips, seeds, order=2, i0=12, eps=0.1)
    for p, s, g in zip(dips, seeds, got):
        assert np.array_equal(g, ps.pwpaintc(p, s, order=2, i0=12, eps=0.1))


def test_pwpaintc_batch_many_sections_across_blocks(ps):
    """48 sections: 96 threads (two per section), so the batch spans two
    64-thread blocks and the section index g / 2 crosses a block boundary."""
    rng = np.random.default_rng(32)
    dips = [(rng.standard_normal((40, 12)) * 1.1).astype(np.float32) for _ in range(48)]
    seeds = [rng.standard_normal(40).astype(np.float32) for _ in range(48)]
    got = ps.pwpaintc_batch(dips, seeds, order=2, i0=5, eps=0.1)
    for p, s, g in zip(dips, seeds, got):
        assert np.array_equal(g, ps.pwpaintc(p, s, order=2, i0=5, eps=0.1))
