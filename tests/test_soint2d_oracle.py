"""The 2-D interpolation's oracle against the reference's own outputs
(golden_soint2d.npz, made by tests/golden/make_golden_soint2d.py from
pyseistr's csoint2d).  The reference's default csoint2d branch is csoint3d's
operator and solver with n3 = 1, so the oracle is the 3-D restatement on a
cube of one slice."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_soint2d.npz")


def _cases():
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    return [(m, z[f"din_{m['k']}"], z[f"mask_{m['k']}"], z[f"dip_{m['k']}"], z[f"out_{m['k']}"])
            for m in meta]


CASES = _cases()


@pytest.mark.parametrize("case", CASES, ids=[f"soint2d-{c[0]['k']}" for c in CASES])
def test_oracle_matches_reference(case):
    m, din, mask, dip, want = case
    if m["twoplane"]:
        # the reference's two-plane branch without preconditioning solves nothing
        assert np.array_equal(want, din)
        return
    got = O.soint3d(din[:, :, None], mask[:, :, None], dip[:, :, None], dip[:, :, None],
                    order=m["order"], niter=m["niter"], njs=tuple(m["njs"]), drift=m["drift"],
                    hasmask=m["hasmask"])[:, :, 0]
    assert np.array_equal(got, want)
