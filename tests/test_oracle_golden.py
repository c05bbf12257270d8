"""The CPU oracle against the reference's own outputs (golden fixtures).

The float32 oracle must reproduce the compiled reference bit for bit; the
FP64 oracle must agree with it to the reference's own float32 accuracy.
"""
import numpy as np
import pytest

from golden_cases import ids, load
from oracle import oracle as O

C2 = load("2d")
C3 = load("3d")


def run_oracle(fn, p, a, precision="f32"):
    if fn == "dip":
        d = a["d"]
        rect = p["rect"]
        mask = a.get("mask")
        if d.ndim == 2:
            return (O.dip2d(d, p["niter"], p["liter"], p["order"], rect, mask=mask,
                            precision=precision),)
        return O.dip3d(d, p["niter"], p["liter"], p["order"], rect, mask=mask, precision=precision)
    if fn == "somean2d":
        return (O.somean2d(a["d"], a["p"], p["ns"], p["order"], p["eps"], p["adj"], precision),)
    if fn == "somf2d":
        return (O.somf2d(a["d"], a["p"], p["ns"], p["order"], p["eps"], p["option"], p["nmf"],
                         precision),)
    if fn == "somean3d":
        return (O.somean3d(a["d"], a["pi"], a["px"], p["r1"], p["r2"], p["order"], precision),)
    if fn == "somf3d":
        return (O.somf3d(a["d"], a["pi"], a["px"], p["r1"], p["r2"], p["order"], p["option"],
                         p["nmf"], precision),)
    if fn == "soint3d":
        return (O.soint3d(a["d"], a["mask"], a["pi"], a["px"], order=p["order"], niter=p["niter"],
                          drift=p["drift"], seed=p["seed"], var=p["var"], precision=precision),)
    raise KeyError(fn)


def expected(a):
    if "out" in a:
        return (a["out"],)
    return a["out_i"], a["out_x"]


@pytest.mark.parametrize("case", C2 + C3, ids=ids(C2) + ids(C3))
def test_oracle_f32_is_bit_exact(case):
    _, fn, p, a = case
    for got, want in zip(run_oracle(fn, p, a), expected(a)):
        assert got.shape == want.shape
        assert np.array_equal(got, want), f"max |diff| {np.abs(got - want).max()}"


def rel_l2(a, b):
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a, np.float64) - b) / (den if den > 0 else 1.0)


@pytest.mark.parametrize("case", [c for c in C2 + C3 if c[1] != "soint3d"],
                         ids=[f"{c[1]}-{c[0]}" for c in C2 + C3 if c[1] != "soint3d"])
def test_oracle_f64_close_to_reference(case):
    """The FP64 oracle differs from the float32 reference only by float rounding."""
    _, fn, p, a = case
    for got, want in zip(run_oracle(fn, p, a, "f64"), expected(a)):
        assert rel_l2(got, want) < 2e-3


DIP_CASES = [c for c in C2 + C3 if c[1] == "dip"]


@pytest.mark.parametrize("case", DIP_CASES, ids=[f"dip-{c[0]}" for c in DIP_CASES])
def test_oracle_gpu_summation_order_on_golden_slopes(case):
    """The oracle's model of the GPU plain path's summation order (GPU_DOTS:
    tile, warp-tree and tile-order sums of float-float dot products) changes
    no slope of the golden cases, on which the GPU plain path is bit-exact
    with the reference; on the full DAS record it moves them 3.7e-2, which
    the GPU matches bit for bit (tests/test_gpu_mixed.py)."""
    _, fn, p, a = case
    d = a["d"]
    mask = a.get("mask")
    if d.ndim == 2:
        got = (O.dip2d(d, p["niter"], p["liter"], p["order"], p["rect"], mask=mask,
                       flags=O.GPU_DOTS),)
    else:
        got = O.dip3d(d, p["niter"], p["liter"], p["order"], p["rect"], mask=mask,
                      flags=O.GPU_DOTS)
    for g, w in zip(got, expected(a)):
        assert np.array_equal(g, w)
