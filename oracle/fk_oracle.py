"""FK dip filter, restated in numpy (the reference's fkdip is numpy too).

TEST INFRASTRUCTURE ONLY: imported by tests/ and by the CPU-baseline leg of
``bench.py``, as the checker or the timed CPU baseline, never by the product
package.

fkdip (pyseistr/fk.py:2-68) passes the part of a section's FK spectrum
inside a cone around k = 0 and returns it in the time-space domain (the DAS
chain subtracts it from the data to remove near-horizontal coherent noise,
demos/test_pyseistr_das.py:50):

1. FFT along time to nf = the next power of two >= n1 samples, keep the
   nf/2 + 1 non-negative frequencies;
2. FFT along space to nk = the next power of two >= n2, k = 0 centred;
3. keep (i1, i2) (1-based, i1 the frequency row, i2 the wavenumber column)
   where i1 > (nf1 / (w nk)) (i2 - nk/2) and i1 > (nf1 / (w nk)) (nk/2 - i2),
   nf1 = nf/2 + 1: a cone of half-width w nk columns at the top row;
4. inverse FFT along space, rebuild the negative frequencies as the complex
   conjugates of rows 1 .. nf/2 - 1 in reverse order, inverse FFT along time,
   real part, cut to n1 x n2.

Precision follows the reference's: the first two FFTs run in the input's
precision (numpy keeps float32 input in complex64), and the float64 mask
promotes the product, so everything after the mask is complex128.  The
comparison products are formed in the reference's order, so cells on the
cone's edge are kept or dropped alike.
"""
from __future__ import annotations

import numpy as np


def pow2_at_least(n: int) -> int:
    """The smallest power of two >= n (1 for n <= 1), as fk.py:138 computes."""
    p = 1
    while p < n:
        p <<= 1
    return p


def cone_mask(nrow: int, nk: int, w: float) -> np.ndarray:
    """The kept cells of the (nrow, nk) shifted FK plane (step 3)."""
    nw = w * nk
    half = nk // 2
    i1 = np.arange(1, nrow + 1, dtype=np.float64)[:, None]
    i2 = np.arange(1, nk + 1, dtype=np.int64)[None, :]
    with np.errstate(divide="ignore", invalid="ignore"):
        s = nrow / nw
        return (i1 > s * (i2 - half)) & (i1 > s * (half - i2))


def fkdip(d, w):
    """The cone-passed part of the 2-D section d (float64 result)."""
    d = np.asarray(d)
    n1, n2 = d.shape
    nf, nk = pow2_at_least(n1), pow2_at_least(n2)
    nrow = nf // 2 + 1
    spec = np.fft.fft(d, nf, axis=0)[:nrow, :]
    fk = np.fft.fftshift(np.fft.fft(spec, nk, axis=1), axes=1)
    fk = fk * cone_mask(nrow, nk, w).astype(np.float64)
    back = np.fft.ifft(np.fft.ifftshift(fk, axes=1), nk, axis=1)
    full = np.zeros((nf, nk), dtype=np.complex128)
    full[:nrow, :] = back
    if nf > 2:
        full[nrow:, :] = np.conj(back[nrow - 2:0:-1, :])
    return np.real(np.fft.ifft(full, nf, axis=0))[:n1, :n2]
