"""The tuning knobs leave the results as they are: the spray's block size
and factor form give the same bits, the mixed CG's axis-1 strip height and
its paired-column kernel only reorder its FP64 dot products (slopes within
1e-5 of the default, each setting deterministic)."""
import os

import numpy as np
import pytest

from gpu_util import need_gpu, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def D():
    need_gpu()
    from pyseistr_gb300 import device

    return device


class _Env:
    def __init__(self, **kv):
        self.kv = {k: v for k, v in kv.items()}

    def __enter__(self):
        self.saved = {k: os.environ.get(k) for k in self.kv}
        for k, v in self.kv.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = str(v)

    def __exit__(self, *exc):
        for k, v in self.saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _secs():
    import workloads

    return [s[: max(64, s.shape[0] // 2), : max(40, s.shape[1] // 3)].copy()
            for s in workloads.batch2d(seed=12, count=6)] + [
        workloads.das2d(n1=300, n2=150, nev=5)]


def _pack(secs):
    import torch

    return torch.from_numpy(np.concatenate([s.reshape(-1, order="F") for s in secs])
                            .astype(np.float32)).cuda()


@pytest.mark.parametrize("strip", [32, 64, 256])
def test_strip_height_reorders_sums_only(D, strip):
    secs = _secs()
    shapes = [s.shape for s in secs]
    d = _pack(secs)
    with _Env(PWD_CG_STRIP=None):
        base = D.dip_batch(d, shapes, 3, 6, 2, (10, 10, 1), mixed=True).cpu().numpy()
    with _Env(PWD_CG_STRIP=strip):
        a = D.dip_batch(d, shapes, 3, 6, 2, (10, 10, 1), mixed=True).cpu().numpy()
        b = D.dip_batch(d, shapes, 3, 6, 2, (10, 10, 1), mixed=True).cpu().numpy()
    assert np.array_equal(a, b)
    assert rel_l2(a, base) <= 1e-5


def test_paired_columns_reorder_sums_only(D):
    """Axis-1 passes with two columns per thread on packed FP32 pairs
    (PWD_CONV1_PAIR=1) against one column per thread (the default): the
    smoothed values are the same per column, only the CG's dot products
    accumulate in another order."""
    secs = _secs() + [np.ascontiguousarray(_secs()[0][:, :37])]  # an odd trace count
    shapes = [s.shape for s in secs]
    d = _pack(secs)
    with _Env(PWD_CONV1_PAIR=None):
        base = D.dip_batch(d, shapes, 3, 6, 2, (10, 10, 1), mixed=True).cpu().numpy()
    with _Env(PWD_CONV1_PAIR="1"):
        a = D.dip_batch(d, shapes, 3, 6, 2, (10, 10, 1), mixed=True).cpu().numpy()
        b = D.dip_batch(d, shapes, 3, 6, 2, (10, 10, 1), mixed=True).cpu().numpy()
    assert np.array_equal(a, b)
    assert rel_l2(a, base) <= 1e-5


def test_paired_columns_odd_trace_length(D):
    """n1 odd: every other row of a strip is not 8-byte aligned and the last
    column pair has one column; the paired kernel agrees with the one-column
    kernel."""
    import workloads

    s = workloads.das2d(n1=333, n2=91, nev=4, seed=9)
    d = _pack([s])
    base = D.dip_batch(d, [s.shape], 3, 6, 2, (10, 10, 1), mixed=True).cpu().numpy()
    with _Env(PWD_CONV1_PAIR="1"):
        a = D.dip_batch(d, [s.shape], 3, 6, 2, (10, 10, 1), mixed=True).cpu().numpy()
    assert rel_l2(a, base) <= 1e-5


@pytest.mark.parametrize("block,split", [(32, None), (64, "1"), (64, "0"), (32, "1")])
def test_spray_knobs_give_the_same_bits(D, block, split):
    secs = _secs()
    shapes = [s.shape for s in secs]
    d = _pack(secs)
    p = D.dip_batch(d, shapes, 2, 4, 2, (10, 10, 1), mixed=True)
    with _Env(PWD_SPRAY_BLOCK=None, PWD_SPRAY_SPLIT=None):
        mean0 = D.sofilter2d_batch(d, p, shapes, 6, 2, 0.01).cpu().numpy()
        med0 = D.sofilter2d_batch(d, p, shapes, 5, 2, 0.01, filter=D.FILTER_MEDIAN).cpu().numpy()
    with _Env(PWD_SPRAY_BLOCK=block, PWD_SPRAY_SPLIT=split):
        mean1 = D.sofilter2d_batch(d, p, shapes, 6, 2, 0.01).cpu().numpy()
        med1 = D.sofilter2d_batch(d, p, shapes, 5, 2, 0.01, filter=D.FILTER_MEDIAN).cpu().numpy()
    assert np.array_equal(mean0, mean1) and np.array_equal(med0, med1)
