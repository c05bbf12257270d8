"""Radon coherence on the GPU (pwd_coherence through cohc / cohc_fb) against
the reference's own outputs (golden_coh.npz) and the oracle: bit for bit,
and, where a curve reaches past the end of the data (the reference reads an
undefined value there; the oracle gives NaN), the value with that sample
read as 0.  The file name sorts after the other GPU tests of the path."""
import json
import os

import numpy as np
import pytest

from coh_util import agrees
from gpu_util import need_gpu

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_coh.npz")


@pytest.fixture(scope="module")
def ps():
    need_gpu()
    import pyseistr_gb300

    return pyseistr_gb300


def test_cohc_fb_matches_reference_in_call_order(ps):
    """The fixture's calls in order, from a fresh hmax state, as the
    reference process made them."""
    from oracle import oracle as O
    from pyseistr_gb300 import api

    z = np.load(GOLDEN)
    api.coh_state.hmax = np.float32(0.0)
    op = O.Coherence()
    for m in json.loads(bytes(z["meta"]).decode()):
        k = m["k"]
        x, v, h = z[f"in_{k}"], z[f"v_{k}"], z[f"h_{k}"]
        got = ps.cohc_fb(x, v, h, m["typ"], m["nt"], v.size, h.size, m["dt"], m["forw"], 0)
        want = op(x, v, h, m["typ"], m["nt"], m["dt"], m["forw"]).reshape(-1, order="F")
        assert got.dtype == np.float32 and got.shape == want.shape
        assert agrees(got, want, x, v, h, m["typ"], m["nt"], m["dt"], op.hmax[0]), k
        ok = ~np.isnan(want)
        assert np.array_equal(got[ok], z[f"out_{k}"][ok]), k
        assert np.isfinite(got).all(), k
    assert api.coh_state.hmax == op.hmax[0]


CASES = [
    # typ, nt, nv, nh, dt, operator, seed, v range, h range
    (1, 1000, 100, 200, 0.0005, -1, 21, (-0.005, 0.005), (0.0, 199.0)),  # a DAS window's shape
    (1, 400, 64, 120, 0.0005, 1, 22, (-0.005, 0.005), (0.0, 119.0)),
    (1, 97, 13, 21, 0.004, 1, 23, (-0.02, 0.03), (-40.0, 60.0)),
    (2, 64, 9, 17, 0.004, -1, 24, (-0.1, 0.2), (-30.0, 50.0)),
    (2, 64, 9, 17, 0.004, 1, 25, (-0.1, 0.2), (-30.0, 50.0)),
    (3, 120, 11, 15, 0.002, -1, 26, (1500.0, 4000.0), (-300.0, 400.0)),
    (3, 120, 11, 15, 0.002, 1, 27, (1500.0, 4000.0), (-300.0, 400.0)),
    (1, 1, 1, 1, 0.004, -1, 28, (0.0, 0.0), (0.0, 0.0)),
]


@pytest.mark.parametrize("case", CASES, ids=[f"typ{c[0]}-{c[1]}x{c[2]}x{c[3]}-op{c[5]}"
                                             for c in CASES])
def test_cohc_matches_oracle(ps, case):
    from oracle import oracle as O
    from pyseistr_gb300 import api

    typ, nt, nv, nh, dt, oper, seed, vr, hr = case
    rng = np.random.default_rng(seed)
    v = np.sort(rng.uniform(*vr, nv)).astype(np.float32)
    h = np.sort(rng.uniform(*hr, nh)).astype(np.float32)
    x = rng.standard_normal((nt, nv if oper == 1 else nh)).astype(np.float32)
    api.coh_state.hmax = np.float32(0.0)
    op = O.Coherence()
    want = op(x, v, h, typ, nt, dt, oper)
    got = ps.cohc(x, {"h": h, "v": v, "nt": nt, "dt": dt, "typ": typ}, operator=oper)
    assert got.shape == (nt, nh if oper == 1 else nv)
    assert agrees(got, want, x, v, h, typ, nt, dt, op.hmax[0])
    assert np.isfinite(got).all()


def test_cohc_device_tensors_and_repeat_calls(ps):
    """A CUDA tensor in gives the same values as a NumPy array in, as a CUDA
    tensor of the reference's shape; repeated calls give the same bits."""
    import torch

    rng = np.random.default_rng(31)
    nt, nh = 300, 48
    v = np.linspace(-0.005, 0.005, 40).astype(np.float32)
    h = np.arange(nh, dtype=np.float32)
    d = rng.standard_normal((nt, nh)).astype(np.float32)
    par = {"h": h, "v": v, "nt": nt, "dt": 0.0005, "typ": 1}
    a = ps.cohc(d, par)
    b = ps.cohc(torch.from_numpy(d).cuda(), par)
    assert isinstance(b, torch.Tensor) and b.is_cuda and tuple(b.shape) == (nt, v.size)
    assert np.array_equal(b.cpu().numpy(), a)
    assert np.array_equal(ps.cohc(d, par), a)


def test_cohc_refuses_what_the_reference_cannot_compute(ps):
    v = np.array([0.0, 1000.0], np.float32)
    h = np.array([5.0, 10.0], np.float32)
    d = np.ones((20, 2), np.float32)
    with pytest.raises(ValueError):  # h / v infinite: no sample index
        ps.cohc(d, {"h": h, "v": v, "nt": 20, "dt": 0.004, "typ": 3})
    with pytest.raises(ValueError):
        ps.cohc_fb(d, v, h, 1, 20, 2, 2, 0.004, 0, 0)
    with pytest.raises(ValueError):  # fewer values than nt * nh
        ps.cohc_fb(d[:10], v, h, 1, 20, 2, 2, 0.004, -1, 0)


def test_cohc_batch_equals_one_call_per_window(ps):
    """The windows of a record in one launch give what one cohc call per
    window gives, adjoint and forward."""
    rng = np.random.default_rng(41)
    nt, nh = 400, 64
    v = np.linspace(-0.005, 0.005, 30).astype(np.float32)
    h = np.arange(nh, dtype=np.float32)
    par = {"h": h, "v": v, "nt": nt, "dt": 0.0005, "typ": 1}
    wins = [rng.standard_normal((nt, nh)).astype(np.float32) for _ in range(5)]
    got = ps.cohc_batch(wins, par)
    for w, g in zip(wins, got):
        assert np.array_equal(g, ps.cohc(w, par))
    models = [rng.standard_normal((nt, v.size)).astype(np.float32) for _ in range(3)]
    got = ps.cohc_batch(models, par, operator=1)
    for m, g in zip(models, got):
        assert np.array_equal(g, ps.cohc(m, par, operator=1))


def test_cohc_batch_parabolic_equals_one_call_per_window(ps):
    """The parabolic type (typ 2) in one launch: its hmax state is the same
    for every window of one offset axis, so the batch equals per-window
    calls, adjoint and forward."""
    rng = np.random.default_rng(43)
    nt, nh = 300, 48
    v = np.linspace(-0.004, 0.004, 24).astype(np.float32)
    h = (np.arange(nh, dtype=np.float32) - 20.0)
    par = {"h": h, "v": v, "nt": nt, "dt": 0.0005, "typ": 2}
    wins = [rng.standard_normal((nt, nh)).astype(np.float32) for _ in range(4)]
    got = ps.cohc_batch(wins, par)
    for w, g in zip(wins, got):
        assert np.array_equal(g, ps.cohc(w, par))
    models = [rng.standard_normal((nt, v.size)).astype(np.float32) for _ in range(3)]
    got = ps.cohc_batch(models, par, operator=1)
    for m, g in zip(models, got):
        assert np.array_equal(g, ps.cohc(m, par, operator=1))
