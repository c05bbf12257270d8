"""Golden fixtures of pyseistr's 2-D structure-oriented interpolation, made by
the reference itself.

Runs the reference's C extension csoint2d (pyseistr/src/soint2d_cfuns.c:2260,
compiled from its own source by ``make -C oracle ref`` into
``oracle/_ref/soint2dcfun*.so``) the way soint2dc (soint2d.py:92-141) calls
it, on small seeded sections with half their traces' samples removed, and
stores inputs, parameters and outputs in tests/golden/golden_soint2d.npz.

    make -C oracle ref && python tests/golden/make_golden_soint2d.py

Cases: PWD orders 1-3, antialiasing step 2, drift (a slope of several
samples), the mask taken from the data (hasmask 0), and the two-plane branch
without preconditioning (which the reference returns unchanged).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))

import soint2dcfun  # noqa: E402

# (n1, n2, order, nj1, niter, drift, hasmask, twoplane, slope scale)
CASES = [
    (80, 40, 1, 1, 20, 0, 1, 0, 0.8),
    (101, 33, 2, 1, 30, 0, 1, 0, 1.2),
    (64, 50, 3, 1, 15, 0, 1, 0, 0.5),
    (90, 30, 2, 2, 20, 0, 1, 0, 0.7),
    (72, 36, 2, 1, 25, 1, 1, 0, 4.0),   # drift: shifts of several samples
    (60, 28, 1, 1, 20, 0, 0, 0, 0.9),   # mask from the data
    (50, 20, 1, 1, 10, 0, 1, 1, 0.6),   # two planes, no preconditioning
]


def section(rng, n1, n2, scale):
    """Seeded dipping events and their local slope (samples per trace)."""
    t = np.arange(n1)[:, None].astype(np.float64)
    x = np.arange(n2)[None, :].astype(np.float64)
    p = scale * np.sin(2 * np.pi * (t / n1 + 0.3 * x / n2))
    shift = np.cumsum(p, axis=1) - p[:, :1]
    d = np.zeros((n1, n2))
    for f0 in (0.05, 0.09, 0.13):
        d += np.cos(2 * np.pi * f0 * (t - shift) + rng.uniform(0, 2 * np.pi))
    d += 0.05 * rng.standard_normal((n1, n2))
    return d.astype(np.float32), p.astype(np.float32)


def main():
    rng = np.random.default_rng(20241207)
    arrays, meta = {}, []
    f = lambda a: np.float32(a).flatten(order="F")  # noqa: E731
    for k, (n1, n2, order, nj1, niter, drift, hasmask, twoplane, scale) in enumerate(CASES):
        d, p = section(rng, n1, n2, scale)
        keep = rng.random(n2) > 0.5  # whole traces missing
        mask = np.repeat(keep[None, :], n1, axis=0).astype(np.float32)
        din = (d * mask).astype(np.float32)
        q = (0.5 * p).astype(np.float32)
        out = soint2dcfun.csoint2d(f(din), f(mask), f(p), f(q if twoplane else p), n1, n2, order,
                                   nj1, nj1, niter, drift, hasmask, twoplane, 0, 0)
        arrays[f"din_{k}"], arrays[f"mask_{k}"] = din, mask
        arrays[f"dip_{k}"] = np.stack([p, q], axis=2) if twoplane else p
        arrays[f"out_{k}"] = np.asarray(out, dtype=np.float32).reshape(n1, n2, order="F")
        meta.append({"k": k, "n1": n1, "n2": n2, "order": order, "njs": [nj1, nj1],
                     "niter": niter, "drift": drift, "hasmask": hasmask, "twoplane": twoplane})
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    path = os.path.join(HERE, "golden_soint2d.npz")
    np.savez_compressed(path, **arrays)
    print(f"wrote {path}: {len(meta)} cases")


if __name__ == "__main__":
    main()
