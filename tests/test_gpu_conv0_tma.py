"""Axis-0 tiles of the mixed CG staged by bulk copies (cp.async.bulk through
an mbarrier: one copy per input array of a tile) against the same kernels
staging element by element with 4-byte cp.async (PWD_CONV0_TMA=0): the
staged values are the same, so the slopes are equal bit for bit, for
traces shorter than a 512-sample segment (several traces per tile), longer
ones (segments with halos), radii compiled in and chosen at run time,
cubes, and an odd CG iteration count.  For cubes, the axis-0 pass of gp
fused into the axis-1 pass that consumes it (k_conv01, the default for
radii 5/5 and 10/10 on the first two axes) gives the bits of the two
separate passes (PWD_CONV01=0)."""
import os

import numpy as np
import pytest

from gpu_util import need_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def D():
    need_gpu()
    from pyseistr_gb300 import device

    return device


def _run(D, secs, niter, liter, rect, tma, fused=True):
    import torch

    env = {"PWD_CONV0_TMA": "1" if tma else "0", "PWD_CONV01": "1" if fused else "0"}
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        shapes = [s.shape for s in secs]
        flat = np.concatenate([s.reshape(-1, order="F") for s in secs]).astype(np.float32)
        return D.dip_batch(torch.from_numpy(flat).cuda(), shapes, niter, liter, 2, rect,
                           mixed=True).cpu().numpy()
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


@pytest.mark.parametrize("rect", [(10, 10, 1), (5, 5, 1), (7, 3, 1), (30, 12, 1), (1, 6, 1)])
def test_bulk_staging_equals_elementwise_staging(D, rect):
    import workloads

    rng = np.random.default_rng(sum(rect))
    secs = [s[: max(64, s.shape[0] // 2), : max(40, s.shape[1] // 4)].copy()
            for s in workloads.batch2d(seed=6, count=5)]
    secs += [rng.standard_normal(sh).astype(np.float32)
             for sh in ((9, 33), (513, 7), (1100, 12), (23, 5), (2000, 9))]
    a = _run(D, secs, 3, 5, rect, True)
    b = _run(D, secs, 3, 5, rect, False)
    assert np.array_equal(a, b)


def test_bulk_staging_with_cubes(D):
    import workloads

    secs = [workloads.plain3d()[:70, :13, :9].copy(), workloads.das2d(n1=300, n2=60, nev=4)]
    a = _run(D, secs, 2, 4, (5, 5, 5), True)
    b = _run(D, secs, 2, 4, (5, 5, 5), False)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("rect", [(5, 5, 5), (10, 10, 4)])
def test_fused_axis0_equals_separate_passes(D, rect):
    import workloads

    rng = np.random.default_rng(70 + sum(rect))
    secs = [s[: max(64, s.shape[0] // 2), : max(40, s.shape[1] // 4)].copy()
            for s in workloads.batch2d(seed=8, count=6)]
    # traces shorter than the axis-0 window, strips with a ragged last one,
    # sections of a single trace pair
    secs += [rng.standard_normal(sh).astype(np.float32)
             for sh in ((7, 30), (9, 33), (70, 5), (513, 7), (1100, 12), (2000, 9), (65, 2))]
    secs += [workloads.plain3d()[:70, :13, :9].copy(),
             rng.standard_normal((40, 11, 6)).astype(np.float32),
             rng.standard_normal((6, 9, 5)).astype(np.float32),
             rng.standard_normal((130, 70, 3)).astype(np.float32)]
    a = _run(D, secs, 3, 5, rect, True, fused=True)
    b = _run(D, secs, 3, 5, rect, True, fused=False)
    assert np.array_equal(a, b)
