"""The FK dip filter oracle against the reference's own outputs
(golden_fk.npz, made by tests/golden/make_golden_fk.py from pyseistr/fk.py)."""
import json
import os

import numpy as np
import pytest

from oracle import fk_oracle as F

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_fk.npz")
Z = np.load(GOLDEN)
META = json.loads(bytes(Z["meta"]).decode())


@pytest.mark.parametrize("m", META, ids=[f"fk-{m['k']}" for m in META])
def test_oracle_matches_reference(m):
    """The same FFT precisions on both sides: equal to 1e-12 of the section's
    amplitude."""
    k = m["k"]
    d, want = Z[f"in_{k}"], Z[f"out_{k}"]
    got = F.fkdip(d, m["w"])
    assert got.shape == want.shape and got.dtype == np.float64
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * float(np.abs(d).max()))


def test_powers_of_two_and_cone():
    assert [F.pow2_at_least(n) for n in (0, 1, 2, 3, 500, 512, 513)] == [1, 1, 2, 4, 512, 512,
                                                                          1024]
    m = F.cone_mask(5, 8, 0.25)  # nk = 8: the centre column is i2 = 4 (0-based 3)
    assert m[:, 3].all()
    assert (m.sum(axis=1)[1:] >= m.sum(axis=1)[:-1]).all()  # widening with frequency


def test_zero_width_raises_like_the_reference():
    with pytest.raises(ZeroDivisionError):
        F.fkdip(np.zeros((8, 8)), 0.0)
