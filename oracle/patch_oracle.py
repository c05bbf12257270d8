"""CPU restatement of pyseistr's patching (pyseistr/patch.py).

TEST INFRASTRUCTURE ONLY: imported by tests/ and the CPU-baseline leg of
``bench.py`` as the checker, never by the product package.

Parity is pinned by tests/golden/golden_patch.npz, made by
tests/golden/make_golden_patch.py from the reference module itself.

The rules restated (patch.py:64-83 patch2d, :178-205 patch3d, :270-304
patch2d_inv, :402-445 patch3d_inv, mode 1):

- each axis of length n is padded with zeros at its end to N = n + s -
  mod(n - l, s) when mod(n - l, s) != 0 (Python's mod: non-negative for a
  positive s, so a window longer than the axis pads it up to l);
- the windows start at 0, s, 2s, ... <= N - l on every axis; the patch id
  runs over the first axis's starts outermost and the last axis's innermost;
- a patch is its window flattened column-major (first axis fastest);
- the inverse adds every patch into a float64 array of the padded size, in
  id order, counts the patches covering each sample, divides, and crops to
  (n1, n2[, n3]).  A sample no window covers (s > l) is 0/0 = NaN.

Outputs here are float32 (the GPU's type): the forward gather is exact, the
inverse is the reference's float64 result rounded once to float32.  The
reference returns float64 when padding occurred (np.zeros is float64) and the
input type otherwise; patch3d returns a trailing axis of length 1.
"""
from __future__ import annotations

import numpy as np


def padded(n: int, l: int, s: int) -> int:
    """Padded axis length (patch.py:66-71)."""
    t = (n - l) % s
    return n + s - t if t != 0 else n


def starts(n: int, l: int, s: int) -> range:
    """Window starts along one axis (patch.py:75-76)."""
    return range(0, padded(n, l, s) - l + 1, s)


def patch(a: np.ndarray, ls, ss) -> np.ndarray:
    """patch2d / patch3d, mode 1: (npatch, prod(ls)) float32."""
    a = np.asarray(a)
    shape = a.shape
    big = np.zeros([padded(n, l, s) for n, l, s in zip(shape, ls, ss)], dtype=np.float64)
    big[tuple(slice(0, n) for n in shape)] = a
    rows = []
    for idx in np.ndindex(*[len(starts(n, l, s)) for n, l, s in zip(shape, ls, ss)]):
        sl = tuple(slice(i * s, i * s + l) for i, l, s in zip(idx, ls, ss))
        rows.append(big[sl].reshape(-1, order="F"))
    return np.asarray(rows, dtype=np.float64).astype(np.float32)


def patch_inv(x: np.ndarray, shape, ls, ss) -> np.ndarray:
    """patch2d_inv / patch3d_inv, mode 1: float32 array of `shape`."""
    x = np.asarray(x, dtype=np.float64).reshape(x.shape[0], -1)
    pshape = [padded(n, l, s) for n, l, s in zip(shape, ls, ss)]
    acc = np.zeros(pshape, dtype=np.float64)
    cnt = np.zeros(pshape, dtype=np.float64)
    k = 0
    for idx in np.ndindex(*[len(starts(n, l, s)) for n, l, s in zip(shape, ls, ss)]):
        sl = tuple(slice(i * s, i * s + l) for i, l, s in zip(idx, ls, ss))
        acc[sl] += x[k].reshape(ls, order="F")
        cnt[sl] += 1.0
        k += 1
    with np.errstate(invalid="ignore", divide="ignore"):
        out = acc / cnt
    return out[tuple(slice(0, n) for n in shape)].astype(np.float32)


def patch2d(a, l1=8, l2=8, s1=4, s2=4):
    return patch(a, (l1, l2), (s1, s2))


def patch3d(a, l1=4, l2=4, l3=4, s1=2, s2=2, s3=2):
    return patch(a, (l1, l2, l3), (s1, s2, s3))


def patch2d_inv(x, n1, n2, l1=8, l2=8, s1=4, s2=4):
    return patch_inv(x, (n1, n2), (l1, l2), (s1, s2))


def patch3d_inv(x, n1, n2, n3, l1=4, l2=4, l3=4, s1=2, s2=2, s3=2):
    return patch_inv(x, (n1, n2, n3), (l1, l2, l3), (s1, s2, s3))
