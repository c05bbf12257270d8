"""2-D structure-oriented interpolation on the GPU (soint2dc / csoint2d
through pwd_soint3d with n3 = 1) against the reference's outputs and the
oracle."""
import json
import os

import numpy as np
import pytest

from gpu_util import need_gpu

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_soint2d.npz")


@pytest.fixture(scope="module")
def ps():
    need_gpu()
    import pyseistr_gb300

    return pyseistr_gb300


def _cases():
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    return [(m, z[f"din_{m['k']}"], z[f"mask_{m['k']}"], z[f"dip_{m['k']}"], z[f"out_{m['k']}"])
            for m in meta]


CASES = _cases()


@pytest.mark.parametrize("case", CASES, ids=[f"soint2d-{c[0]['k']}" for c in CASES])
def test_soint2dc_matches_reference(ps, case):
    m, din, mask, dip, want = case
    got = ps.soint2dc(din, mask, dip, order=m["order"], niter=m["niter"], njs=m["njs"],
                      drift=m["drift"], hasmask=m["hasmask"], twoplane=m["twoplane"], verb=0)
    assert got.shape == want.shape and got.dtype == np.float32
    assert np.array_equal(got, want)


def test_csoint2d_tuple_and_device_tensors(ps):
    """The positional entry on flat arrays, and CUDA tensors in and out."""
    import torch

    m, din, mask, dip, want = CASES[1]
    f = lambda a: np.float32(a).flatten(order="F")  # noqa: E731
    n1, n2 = din.shape
    flat = ps.csoint2d(f(din), f(mask), f(dip), f(dip), n1, n2, m["order"], 1, 1, m["niter"],
                       0, 1, 0, 0, 0)
    assert np.array_equal(flat, f(want))
    t = ps.soint2dc(torch.from_numpy(din).cuda(), torch.from_numpy(mask).cuda(),
                    torch.from_numpy(dip).cuda(), order=m["order"], niter=m["niter"], verb=0)
    assert t.is_cuda and np.array_equal(t.cpu().numpy(), want)


def test_soint2dc_vs_oracle_larger(ps):
    """A 400 x 300 section with a third of its traces missing, order 2."""
    import workloads
    from oracle import oracle as O

    d = workloads.das2d(n1=400, n2=300, nev=5, seed=4)
    rng = np.random.default_rng(8)
    keep = rng.random(300) > 0.33
    mask = np.repeat(keep[None, :], 400, axis=0).astype(np.float32)
    dip = np.full((400, 300), 0.3, np.float32)
    din = (d * mask).astype(np.float32)
    got = ps.soint2dc(din, mask, dip, order=2, niter=25, verb=0)
    want = O.soint3d(din[:, :, None], mask[:, :, None], dip[:, :, None], dip[:, :, None],
                     order=2, niter=25)[:, :, 0]
    assert np.array_equal(got, want)
