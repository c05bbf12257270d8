"""The sparse-data interpolation oracle (csint2d, csint3d) against the
reference's own outputs (golden_sint.npz, made by
tests/golden/make_golden_sint.py from pyseistr's compiled extensions)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_sint.npz")
Z = np.load(GOLDEN)
META = json.loads(bytes(Z["meta"]).decode())


@pytest.mark.parametrize("m", META, ids=[f"{m['dim']}d-{m['k']}" for m in META])
def test_oracle_matches_reference(m):
    k = m["k"]
    if m["dim"] == 2:
        got = O.sint2d(Z[f"d2_{k}"], Z[f"m2_{k}"], Z[f"p2_{k}"], niter=m["niter"], eps=m["eps"],
                       ns=m["ns"], order=m["order"])
        want = Z[f"o2_{k}"]
    else:
        got = O.sint3d(Z[f"d3_{k}"], Z[f"m3_{k}"], Z[f"pi3_{k}"], Z[f"px3_{k}"],
                       niter=m["niter"], eps=m["eps"], ns1=m["ns"][0], ns2=m["ns"][1],
                       order1=m["order"][0], order2=m["order"][1])
        want = Z[f"o3_{k}"]
    assert got.shape == want.shape
    assert np.array_equal(got, want)
