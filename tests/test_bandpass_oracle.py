"""The band-pass oracle against the reference's own outputs (golden_bp.npz,
made by tests/golden/make_golden_bp.py from pyseistr's cbp)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_bp.npz")


def _cases():
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    return [(m, z[f"in_{m['k']}"], z[f"out_{m['k']}"]) for m in meta]


CASES = _cases()


@pytest.mark.parametrize("case", CASES, ids=[f"bp-{c[0]['k']}" for c in CASES])
def test_oracle_matches_reference(case):
    m, a, want = case
    got = O.bandpass(a, m["dt"], m["flo"], m["fhi"], m["nplo"], m["nphi"], m["phase"])
    assert got.shape == want.shape and got.dtype == np.float32
    assert np.array_equal(got, want)


def test_oracle_passes_through_when_no_cut():
    """flo = 0 and fhi at Nyquist: neither filter is applied."""
    a = np.random.default_rng(1).standard_normal((64, 3)).astype(np.float32)
    assert np.array_equal(O.bandpass(a, 0.004, 0.0, 125.0), a)
