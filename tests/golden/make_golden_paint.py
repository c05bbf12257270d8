"""Golden fixtures of pyseistr's plane-wave painting (pwpaintc, rgt), made by
the reference itself.

Runs the reference's C extension cpaint2d (pyseistr/src/paint_cfuns.c:1861,
compiled from its own source by ``make -C oracle ref`` into
``oracle/_ref/paint2dcfun*.so``) the way pwpaintc (rgt.py:57-87) calls it:
rgt's time trace (rgt.py:51) and a seismic trace as seeds, painted from a
reference trace at either end or inside, on seeded slope fields; stored in
tests/golden/golden_paint.npz.

    make -C oracle ref && python tests/golden/make_golden_paint.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))

import paint2dcfun  # noqa: E402

CASES = [  # (n1, n2, order, i0, eps, seed kind, slope amplitude)
    (200, 120, 2, 50, 0.1, "time", 1.5),
    (150, 80, 1, 0, 0.01, "time", 0.8),
    (128, 64, 3, 63, 0.01, "wave", 2.0),
    (100, 90, 2, 45, 0.1, "wave", 3.0),
]


def main():
    rng = np.random.default_rng(20241209)
    arrays, meta = {}, []
    f = lambda a: np.float32(a).flatten(order="F")  # noqa: E731
    for k, (n1, n2, order, i0, eps, kind, amp) in enumerate(CASES):
        t = np.arange(n1)[:, None]
        x = np.arange(n2)[None, :]
        p = amp * np.sin(2 * np.pi * (t / n1 + 0.3 * x / n2)) + 0.1 * rng.standard_normal((n1, n2))
        p = p.astype(np.float32)
        if kind == "time":
            seed = (np.linspace(0, 0.004 * (n1 - 1), n1) - 0.2).astype(np.float32)
        else:
            seed = np.cos(2 * np.pi * 0.05 * np.arange(n1)) * np.exp(-((np.arange(n1) - n1 / 2) /
                                                                      (n1 / 5)) ** 2)
            seed = seed.astype(np.float32)
        out = paint2dcfun.cpaint2d(f(p), seed, n1, n2, order, i0, eps, 0)
        arrays[f"dip_{k}"], arrays[f"seed_{k}"] = p, seed
        arrays[f"out_{k}"] = np.asarray(out, np.float32).reshape(n1, n2, order="F")
        meta.append({"k": k, "order": order, "i0": i0, "eps": eps})
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    path = os.path.join(HERE, "golden_paint.npz")
    np.savez_compressed(path, **arrays)
    print(f"wrote {path}: {len(meta)} cases")


if __name__ == "__main__":
    main()
