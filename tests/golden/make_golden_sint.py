"""Golden fixtures of pyseistr's sparse-data interpolation (sint2dc,
sint3dc), made by the reference itself.

Runs the reference's C extensions csint2d (pyseistr/src/soint2d_cfuns.c:2421)
and csint3d (pyseistr/src/soint3d_cfuns.c:2510), compiled from their own
sources by ``make -C oracle ref`` into ``oracle/_ref/``, the way sint2dc and
sint3dc (sint.py:61-131) call them, on small seeded sections and cubes with
most traces missing, and stores inputs, parameters and outputs in
tests/golden/golden_sint.npz.

    make -C oracle ref && python tests/golden/make_golden_sint.py
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
import soint3dcfun  # noqa: E402

CASES_2D = [  # (n1, n2, niter, ns, order, eps, fraction of traces kept)
    (80, 40, 20, 1, 1, 0.01, 0.3),
    (101, 30, 30, 2, 2, 0.01, 0.2),
    (64, 25, 15, 3, 1, 0.1, 0.4),
    (70, 20, 10, 1, 3, 0.01, 0.25),
]
CASES_3D = [  # (n1, n2, n3, niter, ns1, ns2, order1, order2, eps, fraction kept)
    (40, 10, 8, 8, 1, 1, 1, 1, 0.01, 0.4),
    (48, 12, 9, 10, 2, 1, 2, 1, 0.01, 0.3),
    (32, 8, 6, 6, 1, 2, 1, 3, 0.1, 0.5),
]


def main():
    rng = np.random.default_rng(20241208)
    f = lambda a: np.float32(a).flatten(order="F")  # noqa: E731
    arrays, meta = {}, []
    for k, (n1, n2, niter, ns, order, eps, keep) in enumerate(CASES_2D):
        t = np.arange(n1)[:, None]
        x = np.arange(n2)[None, :]
        p = (0.7 * np.sin(2 * np.pi * (t / n1 + 0.2 * x / n2))).astype(np.float32)
        d = np.cos(2 * np.pi * 0.07 * (t - np.cumsum(p, axis=1))).astype(np.float32)
        mask = np.repeat((rng.random(n2) < keep)[None, :], n1, axis=0).astype(np.float32)
        din = (d * mask).astype(np.float32)
        out = soint2dcfun.csint2d(f(din), f(p), f(mask), n1, n2, niter, ns, order, 0, eps)
        arrays[f"d2_{k}"], arrays[f"m2_{k}"], arrays[f"p2_{k}"] = din, mask, p
        arrays[f"o2_{k}"] = np.asarray(out, np.float32).reshape(n1, n2, order="F")
        meta.append({"dim": 2, "k": k, "niter": niter, "ns": ns, "order": order, "eps": eps})
    for k, (n1, n2, n3, niter, ns1, ns2, o1, o2, eps, keep) in enumerate(CASES_3D):
        pi = rng.uniform(-1, 1, (n1, n2, n3)).astype(np.float32)
        px = rng.uniform(-1, 1, (n1, n2, n3)).astype(np.float32)
        d = rng.standard_normal((n1, n2, n3)).astype(np.float32)
        mask = np.broadcast_to((rng.random((n2, n3)) < keep)[None], (n1, n2, n3))
        mask = mask.astype(np.float32)
        din = (d * mask).astype(np.float32)
        out = soint3dcfun.csint3d(f(din), f(pi), f(px), f(mask), n1, n2, n3, niter, ns1, ns2, o1,
                                  o2, 0, eps)
        arrays[f"d3_{k}"], arrays[f"m3_{k}"] = din, mask
        arrays[f"pi3_{k}"], arrays[f"px3_{k}"] = pi, px
        arrays[f"o3_{k}"] = np.asarray(out, np.float32).reshape(n1, n2, n3, order="F")
        meta.append({"dim": 3, "k": k, "niter": niter, "ns": [ns1, ns2], "order": [o1, o2],
                     "eps": eps})
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    path = os.path.join(HERE, "golden_sint.npz")
    np.savez_compressed(path, **arrays)
    print(f"wrote {path}: {len(meta)} cases")


if __name__ == "__main__":
    main()
