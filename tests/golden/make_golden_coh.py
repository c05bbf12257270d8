"""Golden fixtures of pyseistr's Radon coherence (cohc), made by the reference
itself.

Runs the reference's C extension cohc_fb (pyseistr/src/coh_cfuns.c:415,
compiled from its own source by ``make -C oracle ref`` into
``oracle/_ref/cohcfun*.so``) the way cohc (das.py:92-121) calls it: linear,
parabolic and hyperbolic curves, forward and adjoint, in one process and in
the order stored (the parabolic type keeps a file-scope maximum offset
between calls); stored in tests/golden/golden_coh.npz.  Adjoint samples
whose stack reaches one past the data array hold an undefined value in the
reference; the fixture stores them as they came out and the tests skip them.

    make -C oracle ref && python tests/golden/make_golden_coh.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))

import cohcfun  # noqa: E402

CASES = [  # (typ, nt, nh, nv, dt, forw)
    (1, 200, 30, 20, 0.004, -1),
    (1, 200, 30, 20, 0.004, 1),
    (3, 150, 24, 16, 0.002, -1),
    (3, 150, 24, 16, 0.002, 1),
    (2, 120, 20, 10, 0.004, -1),
    (2, 120, 20, 10, 0.004, 1),
    (1, 300, 48, 31, 0.002, -1),
]


def axes(typ, nh, nv):
    if typ == 1:
        return np.linspace(0, 1, nh), np.linspace(-0.2, 0.2, nv)
    if typ == 2:
        return np.linspace(-300, 500, nh), np.linspace(-0.1, 0.3, nv)
    return np.linspace(-300, 500, nh), np.linspace(1500, 4000, nv)


def main():
    rng = np.random.default_rng(20241210)
    arrays, meta = {}, []
    for k, (typ, nt, nh, nv, dt, forw) in enumerate(CASES):
        h, v = (a.astype(np.float32) for a in axes(typ, nh, nv))
        din = rng.standard_normal(nt * (nh if forw == -1 else nv)).astype(np.float32)
        out = np.asarray(cohcfun.cohc_fb(din, v, h, typ, nt, nv, nh, dt, forw, 0), np.float32)
        arrays[f"in_{k}"], arrays[f"v_{k}"], arrays[f"h_{k}"] = din, v, h
        arrays[f"out_{k}"] = out
        meta.append({"k": k, "typ": typ, "nt": nt, "dt": dt, "forw": forw})
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    path = os.path.join(HERE, "golden_coh.npz")
    np.savez_compressed(path, **arrays)
    print(f"wrote {path}: {len(meta)} cases")


if __name__ == "__main__":
    main()
