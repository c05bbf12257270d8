"""The preconditioned 2-D interpolation's oracle (soint2d_prec in
oracle/pwd_oracle.cpp) against the reference's own outputs
(golden_soint2d_prec.npz, made by tests/golden/make_golden_soint2d_prec.py
from pyseistr's csoint2d with prec = 1): bit for bit."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_soint2d_prec.npz")


def _cases():
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    return [(m, z[f"din_{m['k']}"], z[f"mask_{m['k']}"], z[f"dip_{m['k']}"], z[f"out_{m['k']}"])
            for m in meta]


CASES = _cases()


@pytest.mark.parametrize("case", CASES, ids=[f"prec-{c[0]['k']}" for c in CASES])
def test_oracle_matches_reference(case):
    m, din, mask, dip, want = case
    got = O.soint2d_prec(din, mask, dip, order=m["order"], niter=m["niter"],
                         hasmask=m["hasmask"], twoplane=m["twoplane"])
    assert np.array_equal(got, want)


def test_no_iterations_returns_the_data():
    m, din, mask, dip, want = next(c for c in CASES if c[0]["niter"] == 0)
    assert np.array_equal(want, din)


def test_fp64_instantiation_runs_the_same_algorithm():
    """The double instantiation stays close to the float one where the
    float CG is well behaved (the first golden case), and is exact on the
    trivial case without iterations."""
    m, din, mask, dip, want = CASES[1]
    f64 = O.soint2d_prec(din, mask, dip, order=m["order"], niter=m["niter"],
                         hasmask=m["hasmask"], twoplane=m["twoplane"], precision="f64")
    assert f64.dtype == np.float64
    assert np.linalg.norm(f64 - want) / np.linalg.norm(f64) < 0.5
