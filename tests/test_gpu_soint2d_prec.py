"""The preconditioned 2-D interpolation on the GPU (soint2dc(..., prec=1) /
csoint2d through pwd_soint2d_prec) against the reference's outputs
(golden_soint2d_prec.npz) and the oracle: bit for bit."""
import json
import os

import numpy as np
import pytest

from gpu_util import need_gpu

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_soint2d_prec.npz")


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


@pytest.mark.parametrize("case", CASES, ids=[f"prec-{c[0]['k']}" for c in CASES])
def test_soint2dc_prec_matches_reference(ps, case):
    m, din, mask, dip, want = case
    got = ps.soint2dc(din, mask, dip, order=m["order"], niter=m["niter"],
                      hasmask=m["hasmask"], twoplane=m["twoplane"], prec=1, verb=0)
    assert got.shape == want.shape and got.dtype == np.float32
    assert np.array_equal(got, want)


def test_csoint2d_prec_positional_entry(ps):
    m, din, mask, dip, want = next(c for c in CASES if c[0]["twoplane"])
    f = lambda a: np.float32(a).flatten(order="F")  # noqa: E731
    n1, n2 = din.shape
    flat = ps.csoint2d(f(din), f(mask), f(dip[:, :, 0]), f(dip[:, :, 1]), n1, n2, m["order"], 1, 1,
                       m["niter"], 0, m["hasmask"], 1, 1, 0)
    assert np.array_equal(flat, f(want))


def _section(n1, n2, seed, two):
    import workloads

    d = workloads.das2d(n1=n1, n2=n2, nev=4, seed=seed)
    rng = np.random.default_rng(seed)
    keep = rng.random(n2) > 0.4
    mask = np.repeat(keep[None, :], n1, axis=0).astype(np.float32)
    t = np.arange(n1)[:, None] / n1
    x = np.arange(n2)[None, :] / n2
    p = (0.6 * np.sin(2 * np.pi * (t + 0.5 * x))).astype(np.float32)
    dip = np.stack([p, (0.4 - 0.3 * p).astype(np.float32)], axis=2) if two else p
    return (d * mask).astype(np.float32), mask, dip


@pytest.mark.parametrize("two", [0, 1])
def test_default_size_vs_oracle(ps, two):
    """The reference's demo size, 501 x 100, order 2, 100 iterations."""
    from oracle import oracle as O

    din, mask, dip = _section(501, 100, 11 + two, two)
    got = ps.soint2dc(din, mask, dip, order=2, niter=100, twoplane=two, prec=1, verb=0)
    want = O.soint2d_prec(din, mask, dip, order=2, niter=100, twoplane=two)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("env", [{"PWD_PREC_BUFFERS": "1"}, {"PWD_PREC_BUFFERS": "0"},
                                 {"PWD_PREC_BUFFERS": "0", "PWD_PREC_VEC": "0"}],
                         ids=["one-buffer", "factors-in-place", "all-in-workspace"])
def test_staging_fallbacks_same_bits(ps, env, monkeypatch):
    """One shared-memory factor buffer, the factors read in place, and the
    trace vectors in the workspace give the double-buffered path's bits."""
    m, din, mask, dip, want = CASES[5]
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    got = ps.soint2dc(din, mask, dip, order=m["order"], niter=m["niter"],
                      hasmask=m["hasmask"], twoplane=m["twoplane"], prec=1, verb=0)
    assert np.array_equal(got, want)


def test_long_traces_vs_oracle(ps):
    """Traces too long for shared-memory factor buffers (n1 = 3000, two
    planes, order 3): the factors are read in place."""
    from oracle import oracle as O

    din, mask, dip = _section(3000, 6, 5, 1)
    got = ps.soint2dc(din, mask, dip, order=3, niter=4, twoplane=1, prec=1, verb=0)
    want = O.soint2d_prec(din, mask, dip, order=3, niter=4, twoplane=1)
    assert np.array_equal(got, want)


def test_device_tensors(ps):
    import torch

    m, din, mask, dip, want = CASES[1]
    t = ps.soint2dc(torch.from_numpy(din).cuda(), torch.from_numpy(mask).cuda(),
                    torch.from_numpy(dip).cuda(), order=m["order"], niter=m["niter"], prec=1,
                    verb=0)
    assert t.is_cuda and np.array_equal(t.cpu().numpy(), want)


def test_batch_equals_one_call_per_section(ps):
    """Sections of uneven size in one batch (the shared-memory plan of the
    longest traces serves every section): every section gets its own call's
    bits, for one and two slope planes."""
    import torch
    from pyseistr_gb300 import device as D

    shapes = [(120, 30), (77, 19), (501, 40), (64, 64), (2, 9), (250, 12)]
    for two in (0, 1):
        secs = [_section(n1, n2, 40 + k, two) for k, (n1, n2) in enumerate(shapes)]
        f = lambda a: torch.from_numpy(  # noqa: E731
            np.concatenate([np.float32(x).reshape(-1, order="F") for x in a])).cuda()
        data, mask = f([s[0] for s in secs]), f([s[1] for s in secs])
        d1 = f([s[2][:, :, 0] if two else s[2] for s in secs])
        d2 = f([s[2][:, :, 1] for s in secs]) if two else None
        got = D.soint2d_prec_batch(data, mask, d1, d2, shapes, order=2, niter=15,
                                   twoplane=two).cpu().numpy()
        k = 0
        for (din, m, dip), (n1, n2) in zip(secs, shapes):
            want = ps.soint2dc(din, m, dip, order=2, niter=15, twoplane=two, prec=1, verb=0)
            assert np.array_equal(got[k:k + n1 * n2], np.float32(want).reshape(-1, order="F"))
            k += n1 * n2


def test_soint2dc_batch_api(ps):
    """The list form against the golden fixtures of one and two planes."""
    for two in (0, 1):
        cases = [c for c in CASES if c[0]["twoplane"] == two and c[0]["order"] == 2]
        got = ps.soint2dc_batch([c[1] for c in cases], [c[2] for c in cases],
                                [c[3] for c in cases], order=2,
                                niter=cases[0][0]["niter"], twoplane=two)
        for c, g in zip(cases, got):
            if c[0]["niter"] == cases[0][0]["niter"] and c[0]["hasmask"] == 1:
                assert np.array_equal(g, c[4])
