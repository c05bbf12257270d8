"""The Radon coherence oracle (cohc_fb) against the reference's own outputs
(golden_coh.npz, made by tests/golden/make_golden_coh.py)."""
import json
import os

import numpy as np

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_coh.npz")


def test_oracle_matches_reference_in_call_order():
    """Replayed in the fixture's order with one operator object, so that the
    parabolic type's carried maximum offset is the reference's; samples the
    reference leaves undefined (NaN from the oracle) are skipped."""
    z = np.load(GOLDEN)
    op = O.Coherence()
    undefined = 0
    for m in json.loads(bytes(z["meta"]).decode()):
        k = m["k"]
        got = op(z[f"in_{k}"], z[f"v_{k}"], z[f"h_{k}"], m["typ"], m["nt"], m["dt"], m["forw"])
        got = got.reshape(-1, order="F")
        want = z[f"out_{k}"]
        bad = np.isnan(got)
        if m["forw"] == 1:
            assert not bad.any()
        undefined += int(bad.sum())
        assert bad.mean() < 0.02
        assert np.array_equal(got[~bad], want[~bad])
    assert undefined > 0  # the past-the-end read is met in practice


def test_forward_and_adjoint_shapes():
    op = O.Coherence()
    h = np.linspace(0, 1, 8).astype(np.float32)
    v = np.linspace(-0.1, 0.1, 5).astype(np.float32)
    m = np.random.default_rng(0).standard_normal((50, 5)).astype(np.float32)
    d = op(m, v, h, 1, 50, 0.004, 1)
    assert d.shape == (50, 8)
    assert op(d, v, h, 1, 50, 0.004, -1).shape == (50, 5)
