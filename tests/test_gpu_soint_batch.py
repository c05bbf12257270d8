"""Batched 3-D interpolation (pwd_soint3d_batch): one launch sequence for
many patches gives every patch the result of its own pwd_soint3d call, and
chains with pwd_dip_batch's slope layout."""
import numpy as np
import pytest

from gpu_util import need_gpu, rel_l2

pytestmark = pytest.mark.gpu


def _pack(arrs):
    return np.concatenate([a.reshape(-1, order="F") for a in arrs]).astype(np.float32)


@pytest.mark.parametrize("drift", [0, 1])
def test_soint3d_batch_equals_per_patch(drift):
    need_gpu()
    import torch
    import workloads
    from pyseistr_gb300 import device as D

    pairs = workloads.patches3d(seed=5, count=4, n1_range=(64, 96), n23_range=(10, 16))
    shapes = [d.shape for d, _ in pairs]
    data = torch.from_numpy(_pack([d for d, _ in pairs])).cuda()
    mask = torch.from_numpy(_pack([m for _, m in pairs])).cuda()
    dips = D.dip_batch(data, shapes, 2, 4, 2, (3, 3, 3))
    dm = data * mask
    out = D.soint3d_batch(dm, mask, dips, shapes, order=2, niter=8, drift=drift).cpu().numpy()
    off = po = 0
    for n1, n2, n3 in shapes:
        n = n1 * n2 * n3
        one = D.soint3d(dm[off:off + n], mask[off:off + n], dips[po:po + n],
                        dips[po + n:po + 2 * n], n1, n2, n3, order=2, niter=8,
                        drift=drift).cpu().numpy()
        assert np.array_equal(out[off:off + n], one)
        off += n
        po += 2 * n


def test_soint3d_batch_vs_oracle():
    """Each patch of a batch against the float oracle's csoint3d."""
    need_gpu()
    import torch
    import workloads
    from oracle import oracle as O
    from pyseistr_gb300 import device as D

    pairs = workloads.patches3d(seed=9, count=3, n1_range=(48, 64), n23_range=(8, 12))
    shapes = [d.shape for d, _ in pairs]
    rng = np.random.default_rng(0)
    dipl = [rng.uniform(-1, 1, d.shape).astype(np.float32) for d, _ in pairs]
    dipx = [rng.uniform(-1, 1, d.shape).astype(np.float32) for d, _ in pairs]
    packed = np.concatenate([np.concatenate([a.reshape(-1, order="F"), b.reshape(-1, order="F")])
                             for a, b in zip(dipl, dipx)])
    dm = _pack([d * m for d, m in pairs])
    mask = _pack([m for _, m in pairs])
    out = D.soint3d_batch(torch.from_numpy(dm).cuda(), torch.from_numpy(mask).cuda(),
                          torch.from_numpy(packed).cuda(), shapes, order=2, niter=10).cpu().numpy()
    off = 0
    for (d, m), a, b in zip(pairs, dipl, dipx):
        want = O.soint3d(d * m, m, a, b, order=2, niter=10).reshape(-1, order="F")
        got = out[off:off + d.size]
        assert rel_l2(got, want) <= 1e-5
        off += d.size


def test_packed_dip_soint3d_equals_device_calls():
    need_gpu()
    import torch
    import workloads
    import pyseistr_gb300 as ps
    from pyseistr_gb300 import device as D

    pairs = workloads.patches3d(seed=13, count=3, n1_range=(48, 64), n23_range=(8, 12))
    shapes = [d.shape for d, _ in pairs]
    data = torch.from_numpy(_pack([d for d, _ in pairs])).pin_memory()
    mask = torch.from_numpy(_pack([m for _, m in pairs])).pin_memory()
    got = ps.dip_soint3d_packed(data, mask, shapes, 2, 4, 2, [3, 3, 3], 2, 6).numpy()
    dd, mm = data.cuda(), mask.cuda()
    dips = D.dip_batch(dd, shapes, 2, 4, 2, (3, 3, 3))
    want = D.soint3d_batch(dd * mm, mm, dips, shapes, order=2, niter=6).cpu().numpy()
    assert np.array_equal(got, want)
