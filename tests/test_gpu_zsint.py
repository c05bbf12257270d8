"""Sparse-data interpolation on the GPU (pwd_sint2d through sint2dc /
csint2d) against the reference's own outputs (golden_sint.npz) and the
oracle.  Every float operation is the reference's; the FP64 dot products are
summed in another order, so the results are expected bit for bit and held
to the stated 1e-4 relative L2.  The file name sorts after the other GPU
tests of the path."""
import json
import os

import numpy as np
import pytest

from gpu_util import DIP_TOL, need_gpu, rel_l2

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_sint.npz")


@pytest.fixture(scope="module")
def ps():
    need_gpu()
    import pyseistr_gb300

    return pyseistr_gb300


def test_sint2dc_matches_reference(ps):
    z = np.load(GOLDEN)
    for m in json.loads(bytes(z["meta"]).decode()):
        if m["dim"] != 2:
            continue
        k = m["k"]
        got = ps.sint2dc(z[f"d2_{k}"], z[f"m2_{k}"], z[f"p2_{k}"], niter=m["niter"], eps=m["eps"],
                         ns=m["ns"], order=m["order"])
        want = z[f"o2_{k}"]
        assert got.dtype == np.float32 and got.shape == want.shape
        assert rel_l2(got, want) <= DIP_TOL, k


CASES = [
    # n1, n2, niter, ns, order, eps, known fraction, seed
    (501, 100, 30, 2, 2, 0.01, 0.3, 11),
    (120, 40, 25, 2, 2, 0.01, 0.3, 12),
    (64, 30, 40, 1, 4, 0.05, 0.5, 13),
    (50, 12, 5, 0, 1, 0.01, 0.2, 14),
    (40, 10, 10, 2, 2, 0.01, 1.0, 15),
    (40, 10, 10, 2, 2, 0.01, 0.0, 16),
    (40, 10, 0, 1, 1, 0.01, 0.4, 17),
]


def _case(n1, n2, frac, seed):
    rng = np.random.default_rng(seed)
    keep = (rng.random(n2) < frac).astype(np.float32)
    mask = np.repeat(keep[None, :], n1, 0)
    d = (rng.standard_normal((n1, n2)) * mask).astype(np.float32)
    dip = (rng.standard_normal((n1, n2)) * 0.7).astype(np.float32)
    return d, mask, dip


@pytest.mark.parametrize("case", CASES, ids=[f"sint2d-{c[0]}x{c[1]}-it{c[2]}-ns{c[3]}-o{c[4]}"
                                             for c in CASES])
def test_sint2dc_matches_oracle(ps, case):
    from oracle import oracle as O

    n1, n2, niter, ns, order, eps, frac, seed = case
    d, mask, dip = _case(n1, n2, frac, seed)
    want = O.sint2d(d, mask, dip, niter=niter, eps=eps, ns=ns, order=order)
    got = ps.sint2dc(d, mask, dip, niter=niter, eps=eps, ns=ns, order=order)
    assert rel_l2(got, want) <= DIP_TOL


def test_sint2dc_device_tensors_and_repeat_calls(ps):
    import torch

    d, mask, dip = _case(80, 24, 0.4, 21)
    a = ps.sint2dc(d, mask, dip, niter=12, ns=2, order=2)
    b = ps.sint2dc(torch.from_numpy(d).cuda(), torch.from_numpy(mask).cuda(),
                   torch.from_numpy(dip).cuda(), niter=12, ns=2, order=2)
    assert isinstance(b, torch.Tensor) and b.is_cuda and tuple(b.shape) == (80, 24)
    assert np.array_equal(b.cpu().numpy(), a)
    assert np.array_equal(ps.sint2dc(d, mask, dip, niter=12, ns=2, order=2), a)


def test_csint2d_refuses_bad_arguments(ps):
    d = np.zeros(40 * 10, np.float32)
    with pytest.raises(ValueError):  # dimension mismatch
        ps.csint2d(d, d, d, 40, 11, 5, 1, 1, 0, 0.01)
    with pytest.raises(ValueError):  # short mask
        ps.csint2d(d, d, d[:100], 40, 10, 5, 1, 1, 0, 0.01)


def test_sint3dc_matches_reference(ps):
    z = np.load(GOLDEN)
    for m in json.loads(bytes(z["meta"]).decode()):
        if m["dim"] != 3:
            continue
        k = m["k"]
        got = ps.sint3dc(z[f"d3_{k}"], z[f"m3_{k}"], z[f"pi3_{k}"], z[f"px3_{k}"],
                         niter=m["niter"], eps=m["eps"], ns1=m["ns"][0], ns2=m["ns"][1],
                         order1=m["order"][0], order2=m["order"][1])
        want = z[f"o3_{k}"]
        assert got.dtype == np.float32 and got.shape == want.shape
        assert rel_l2(got, want) <= DIP_TOL, k


CASES3 = [
    # n1, n2, n3, niter, (ns1, ns2), (order1, order2), eps, known fraction, seed
    (64, 20, 16, 10, (2, 2), (2, 2), 0.01, 0.5, 31),
    (40, 9, 7, 8, (1, 2), (2, 1), 0.01, 0.3, 32),
    (24, 5, 11, 12, (2, 1), (1, 3), 0.05, 0.5, 33),
    (16, 6, 1, 6, (2, 2), (2, 2), 0.01, 0.4, 34),
    (16, 1, 6, 6, (1, 1), (2, 2), 0.01, 0.4, 35),
]


def _case3(n1, n2, n3, frac, seed):
    rng = np.random.default_rng(seed)
    keep = (rng.random((n2, n3)) < frac).astype(np.float32)
    mask = np.repeat(keep[None], n1, 0)
    d = (rng.standard_normal((n1, n2, n3)) * mask).astype(np.float32)
    pi = (rng.standard_normal((n1, n2, n3)) * 0.6).astype(np.float32)
    px = (rng.standard_normal((n1, n2, n3)) * 0.6).astype(np.float32)
    return d, mask, pi, px


@pytest.mark.parametrize("case", CASES3, ids=[f"sint3d-{c[0]}x{c[1]}x{c[2]}-it{c[3]}"
                                              for c in CASES3])
def test_sint3dc_matches_oracle(ps, case):
    from oracle import oracle as O

    n1, n2, n3, niter, ns, order, eps, frac, seed = case
    d, mask, pi, px = _case3(n1, n2, n3, frac, seed)
    want = O.sint3d(d, mask, pi, px, niter=niter, eps=eps, ns1=ns[0], ns2=ns[1], order1=order[0],
                    order2=order[1])
    got = ps.sint3dc(d, mask, pi, px, niter=niter, eps=eps, ns1=ns[0], ns2=ns[1],
                     order1=order[0], order2=order[1])
    assert rel_l2(got, want) <= DIP_TOL
