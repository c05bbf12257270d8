"""Band-pass on the GPU (pwd_bandpass) against the reference's outputs and
the oracle (which is pinned bit for bit to the reference's cbp)."""
import json
import os

import numpy as np
import pytest

from gpu_util import need_gpu

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_bp.npz")


@pytest.fixture(scope="module")
def ps():
    need_gpu()
    import pyseistr_gb300

    return pyseistr_gb300


def _cases():
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    return [(m, z[f"in_{m['k']}"], z[f"out_{m['k']}"]) for m in meta]


CASES = _cases()


@pytest.mark.parametrize("case", CASES, ids=[f"bp-{c[0]['k']}" for c in CASES])
def test_bandpass_matches_reference(ps, case):
    """Bit for bit against the oracle run on this host; against the fixtures
    (made on another host, whose C library's sinf / cosf may round a
    coefficient differently) to 1e-5 of the trace amplitude."""
    from oracle import oracle as O

    m, a, want = case
    args = (m["dt"], m["flo"], m["fhi"], m["nplo"], m["nphi"], m["phase"])
    got = ps.bandpassc(a, *args, verb=0)
    exp_shape = want.shape if want.ndim == 3 else np.squeeze(want).shape
    assert got.shape == exp_shape and got.dtype == np.float32
    assert np.array_equal(got, np.squeeze(O.bandpass(a, *args)) if want.ndim < 3
                          else O.bandpass(a, *args))
    np.testing.assert_allclose(got, np.squeeze(want) if want.ndim < 3 else want, rtol=0,
                               atol=1e-5 * float(np.abs(want).max()))


@pytest.mark.parametrize("shape,args", [
    ((2000, 77), (0.0005, 0.0, 200.0, 6, 6, 0)),      # the DAS demo's filter
    ((1001, 45), (0.004, 4.0, 60.0, 6, 6, 0)),        # both cuts, partial chunk
    ((333, 33), (0.002, 10.0, 90.0, 5, 9, 1)),        # minimum phase, odd poles
    ((64, 40), (0.004, 3.0, 100.0, 30, 30, 0)),       # 12 passes: two launches
    ((31, 3), (0.004, 5.0, 40.0, 20, 2, 0)),          # trace shorter than a chunk
    ((90, 7, 6), (0.004, -0.02, -0.3, 4, 4, 0)),      # negative cut-offs
])
def test_bandpass_vs_oracle(ps, shape, args):
    from oracle import oracle as O

    a = np.random.default_rng(3).standard_normal(shape).astype(np.float32)
    got = ps.bandpassc(a, *args, verb=0)
    want = O.bandpass(a, *args)
    # a negative high cut makes an unstable filter: overflow and NaN alike
    assert np.array_equal(got, np.squeeze(want) if len(shape) < 3 else want, equal_nan=True)


def test_bandpass_das_record_on_device(ps):
    """The full 2000 x 5000 DAS record with the demo's filter, device in and
    out, in place: every trace equal to the oracle's."""
    import torch
    import workloads
    from oracle import oracle as O
    from pyseistr_gb300 import device as D

    d = workloads.das2d(seed=5)
    t = torch.from_numpy(np.asfortranarray(d).reshape(-1, order="F").copy()).cuda()
    D.bandpass(t, (2000, 5000, 1), 0.0005, 0.0, 200.0, 6, 6, 0, out=t)
    got = t.cpu().numpy().reshape(2000, 5000, order="F")
    assert np.array_equal(got, O.bandpass(d, 0.0005, 0.0, 200.0, 6, 6, 0))


def test_traces_are_independent(ps):
    """A subset of traces filters to the same values as inside the record."""
    import workloads

    d = workloads.das2d(n1=700, n2=300, nev=5, seed=2)
    full = ps.bandpassc(d, 0.001, 2.0, 150.0, 6, 6, 0, verb=0)
    part = ps.bandpassc(np.ascontiguousarray(d[:, 37:101]), 0.001, 2.0, 150.0, 6, 6, 0, verb=0)
    assert np.array_equal(full[:, 37:101], part)


def test_shapes_and_pass_through(ps, capsys):
    a = np.random.default_rng(4).standard_normal(200).astype(np.float32)
    one = ps.bandpassc(a, 0.004, 0, 20, verb=0)
    assert one.shape == (200,)
    col = ps.bandpassc(a[:, None], 0.004, 0, 20, verb=0)
    assert np.array_equal(one, col)
    # no cut at all: the input comes back
    assert np.array_equal(ps.bandpassc(a, 0.004, 0, 125.0, verb=0), a)
    with pytest.raises(ValueError):
        ps.bandpassc(a[None, :], 0.004, 0, 20, verb=0)
    ps.bandpassc(a, 0.004, 30, 20, verb=1)
    out = capsys.readouterr().out
    assert "Need flo < fhi" in out and "nplo=6,n123=200" in out
