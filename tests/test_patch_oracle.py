"""The patching oracle against the reference's own outputs (golden_patch.npz,
made by tests/golden/make_golden_patch.py from pyseistr/patch.py)."""
import json
import os

import numpy as np
import pytest

from oracle import patch_oracle as P

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_patch.npz")


def _cases():
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    return [(m, z[f"a{m['dim']}_{m['k']}"], z[f"x{m['dim']}_{m['k']}"],
             z[f"b{m['dim']}_{m['k']}"]) for m in meta]


CASES = _cases()


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]['dim']}d-{c[0]['k']}" for c in CASES])
def test_oracle_matches_reference(case):
    """Patches bit for bit; the inverse equal to the reference's float64
    result rounded to float32 (NaN where no window covers a sample)."""
    m, a, x, b = case
    xr = x[:, :, 0] if m["dim"] == 3 else x
    got = P.patch(a, m["l"], m["s"])
    assert got.shape == xr.shape
    assert np.array_equal(got, xr.astype(np.float32))
    inv = P.patch_inv(xr, m["n"], m["l"], m["s"])
    assert np.array_equal(inv, b.astype(np.float32), equal_nan=True)


@pytest.mark.parametrize("shape,l,s", [((13, 10, 9), (4, 4, 4), (2, 2, 2)),
                                       ((12, 11, 9), (4, 4, 4), (2, 2, 2))])
def test_oracle_3d_patterns_the_reference_leaves_unassigned(shape, l, s):
    """Axes 1 and 3 padded but not 2, or 2 and 3 but not 1: the reference's
    patch3d_inv raises; the oracle pads every axis alike and round-trips."""
    a = np.random.default_rng(3).standard_normal(shape).astype(np.float32)
    assert np.array_equal(P.patch_inv(P.patch(a, l, s), shape, l, s), a)


def test_padding_lengths():
    assert P.padded(37, 8, 4) == 40 and P.padded(32, 8, 4) == 32
    assert P.padded(5, 8, 4) == 8  # window longer than the axis
    assert len(P.starts(37, 8, 4)) == 9
