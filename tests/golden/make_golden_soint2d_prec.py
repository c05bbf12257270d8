"""Golden fixtures of pyseistr's preconditioned 2-D structure-oriented
interpolation (soint2dc(..., prec=1)), made by the reference itself.

Runs the reference's C extension csoint2d (pyseistr/src/soint2d_cfuns.c:2260,
prec = 1 branches :2354-2398, compiled from its own source by
``make -C oracle ref`` into ``oracle/_ref/soint2dcfun*.so``) the way soint2dc
(soint2d.py:92-141) calls it, on small seeded sections with traces or
scattered samples removed, and stores inputs, parameters and outputs in
tests/golden/golden_soint2d_prec.npz.

    make -C oracle ref && python tests/golden/make_golden_soint2d_prec.py

Cases: PWD orders 1-3, one and two slope planes (predict_lop and
predict2_lop), the mask taken from the data (hasmask 0), scattered missing
samples, no iterations (the data returned), and tiny traces (n1 = 2, 5).
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

# (n1, n2, order, niter, hasmask, twoplane, slope scale, mask kind)
CASES = [
    (80, 40, 1, 20, 1, 0, 0.8, "traces"),
    (101, 33, 2, 30, 1, 0, 1.2, "traces"),
    (64, 50, 3, 15, 1, 0, 0.5, "traces"),
    (60, 28, 1, 20, 0, 0, 0.9, "traces"),    # mask from the data
    (50, 20, 1, 10, 1, 1, 0.6, "traces"),    # two planes
    (72, 36, 2, 25, 1, 1, 1.0, "traces"),
    (90, 24, 2, 20, 1, 1, 0.7, "samples"),   # two planes, scattered samples
    (70, 30, 2, 40, 1, 0, 0.9, "samples"),
    (40, 12, 2, 0, 1, 0, 0.5, "traces"),     # no iterations
    (5, 7, 1, 10, 1, 0, 0.3, "traces"),
    (2, 9, 1, 6, 1, 0, 0.3, "samples"),
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
    rng = np.random.default_rng(20261204)
    arrays, meta = {}, []
    f = lambda a: np.float32(a).flatten(order="F")  # noqa: E731
    for k, (n1, n2, order, niter, hasmask, twoplane, scale, kind) in enumerate(CASES):
        d, p = section(rng, n1, n2, scale)
        if kind == "traces":
            keep = rng.random(n2) > 0.5
            mask = np.repeat(keep[None, :], n1, axis=0).astype(np.float32)
        else:
            mask = (rng.random((n1, n2)) > 0.4).astype(np.float32)
        din = (d * mask).astype(np.float32)
        q = (0.5 * p + 0.1).astype(np.float32)
        out = soint2dcfun.csoint2d(f(din), f(mask), f(p), f(q if twoplane else p), n1, n2, order,
                                   1, 1, niter, 0, hasmask, twoplane, 1, 0)
        arrays[f"din_{k}"], arrays[f"mask_{k}"] = din, mask
        arrays[f"dip_{k}"] = np.stack([p, q], axis=2) if twoplane else p
        arrays[f"out_{k}"] = np.asarray(out, dtype=np.float32).reshape(n1, n2, order="F")
        meta.append({"k": k, "n1": n1, "n2": n2, "order": order, "niter": niter,
                     "hasmask": hasmask, "twoplane": twoplane})
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    path = os.path.join(HERE, "golden_soint2d_prec.npz")
    np.savez_compressed(path, **arrays)
    print(f"wrote {path}: {len(meta)} cases")


if __name__ == "__main__":
    main()
