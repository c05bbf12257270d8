"""The plane-wave painting oracle (cpaint2d) against the reference's own
outputs (golden_paint.npz, made by tests/golden/make_golden_paint.py)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_paint.npz")
Z = np.load(GOLDEN)
META = json.loads(bytes(Z["meta"]).decode())


@pytest.mark.parametrize("m", META, ids=[f"paint-{m['k']}" for m in META])
def test_oracle_matches_reference(m):
    k = m["k"]
    got = O.paint2d(Z[f"dip_{k}"], Z[f"seed_{k}"], order=m["order"], i0=m["i0"], eps=m["eps"])
    assert np.array_equal(got, Z[f"out_{k}"])
    # the reference trace is the seed itself
    assert np.array_equal(got[:, m["i0"]], Z[f"seed_{k}"])


def test_reference_trace_out_of_range_is_refused():
    with pytest.raises(ValueError):
        O.paint2d(np.zeros((16, 4), np.float32), np.zeros(16, np.float32), i0=4)
