"""Patching on the GPU (pwd_patch / pwd_patch_inv) against the reference's
outputs, the oracle, and size-independent properties."""
import json
import os

import numpy as np
import pytest

from gpu_util import need_gpu

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_patch.npz")


@pytest.fixture(scope="module")
def ps():
    need_gpu()
    import pyseistr_gb300

    return pyseistr_gb300


def _cases():
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    return [(m, z[f"a{m['dim']}_{m['k']}"], z[f"x{m['dim']}_{m['k']}"],
             z[f"b{m['dim']}_{m['k']}"]) for m in meta]


CASES = _cases()


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]['dim']}d-{c[0]['k']}" for c in CASES])
def test_patch_matches_reference(ps, case):
    m, a, x, b = case
    if m["dim"] == 2:
        got = ps.patch2d(a, *m["l"], *m["s"])
        inv = ps.patch2d_inv(x, *m["n"], *m["l"], *m["s"])
    else:
        got = ps.patch3d(a, *m["l"], *m["s"])
        inv = ps.patch3d_inv(x, *m["n"], *m["l"], *m["s"])
    assert got.shape == x.shape and got.dtype == np.float32
    assert np.array_equal(got, x.astype(np.float32))
    assert np.array_equal(inv, b.astype(np.float32), equal_nan=True)


@pytest.mark.parametrize("shape,l,s", [((13, 10, 9), (4, 4, 4), (2, 2, 2)),
                                       ((12, 11, 9), (4, 4, 4), (2, 2, 2)),
                                       ((3, 40, 7), (4, 8, 2), (2, 6, 3)),
                                       ((101, 1, 1), (16, 1, 1), (5, 1, 1))])
def test_patch3d_vs_oracle(ps, shape, l, s):
    from oracle import patch_oracle as P

    a = np.random.default_rng(7).standard_normal(shape).astype(np.float32)
    x = ps.patch3d(a, *l, *s)
    assert np.array_equal(x[:, :, 0], P.patch(a, l, s))
    xs = (x[:, :, 0] * 1.5 - 0.25).astype(np.float32)  # distinct patch values
    assert np.array_equal(ps.patch3d_inv(xs, *shape, *l, *s),
                          P.patch_inv(xs, shape, l, s), equal_nan=True)


def test_round_trip_das_record(ps):
    """Full configuration-3 size (2000 x 5000, 64 x 64 windows at stride 32):
    the inverse of the patches is the record, bit for bit, on the device."""
    import torch
    import workloads

    d = torch.from_numpy(workloads.das2d(seed=5)).cuda()
    x = ps.patch2d(d, 64, 64, 32, 32)
    from oracle import patch_oracle as P

    npatch = len(P.starts(2000, 64, 32)) * len(P.starts(5000, 64, 32))
    assert x.is_cuda and tuple(x.shape) == (npatch, 64 * 64)
    back = ps.patch2d_inv(x, 2000, 5000, 64, 64, 32, 32)
    assert torch.equal(back, d)


def test_patches_feed_the_batched_slope_estimation(ps):
    """The patch matrix is the packed-section layout: its rows, as a batch of
    64 x 48 sections, give each patch's dip2dc slopes bit for bit."""
    import torch
    import workloads
    from pyseistr_gb300 import device as D

    d = workloads.das2d(n1=300, n2=200, nev=6, seed=9)
    x = ps.patch2d(torch.from_numpy(d).cuda(), 64, 48, 32, 24)
    shapes = [(64, 48)] * x.shape[0]
    slopes = D.dip_batch(x.reshape(-1), shapes, 2, 4, 2, (5, 5, 1)).view(x.shape).cpu().numpy()
    xh = x.cpu().numpy()
    for k in (0, 7, x.shape[0] - 1):
        one = ps.dip2dc(xh[k].reshape(64, 48, order="F"), niter=2, liter=4, order=2,
                        rect=[5, 5, 1])
        assert np.array_equal(slopes[k].reshape(64, 48, order="F"), one)


def test_invalid_sizes(ps):
    with pytest.raises(ValueError):
        ps.patch2d(np.zeros((8, 8), np.float32), 0, 4, 2, 2)
    with pytest.raises(ValueError):
        ps.patch2d(np.zeros((8, 8), np.float32), mode=2)
    # a window longer than an axis whose excess the stride divides: the
    # reference's window loop is empty (no patches); refused here
    with pytest.raises(ValueError):
        ps.patch3d(np.zeros((3, 40, 7), np.float32), 5, 8, 2, 2, 6, 3)
