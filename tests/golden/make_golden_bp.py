"""Golden fixtures of pyseistr's band-pass, made by the reference itself.

Runs the reference's C extension cbp (pyseistr/src/bp_cfuns.c, compiled from
its own source by ``make -C oracle ref`` into ``oracle/_ref/bpcfun*.so``) on
small seeded traces the way bandpassc (bp.py:128-181) calls it, and stores
inputs, parameters and outputs in tests/golden/golden_bp.npz.

    make -C oracle ref && python tests/golden/make_golden_bp.py

Cases: zero and minimum phase, low-cut only, high-cut only, both, odd and
even pole counts (first-order sections), one pole, cut-offs at the edges of
the accepted range, a 3-D array and a single trace.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
sys.path.insert(0, ROOT)

import bpcfun  # noqa: E402

import workloads as W  # noqa: E402

# (shape, dt, flo, fhi, nplo, nphi, phase)
CASES = [
    ((500, 40), 0.004, 5.0, 40.0, 6, 6, 0),
    ((500, 40), 0.004, 5.0, 40.0, 6, 6, 1),
    ((333, 17), 0.002, 0.0, 60.0, 6, 6, 0),      # high cut only
    ((333, 17), 0.002, 10.0, 250.0, 6, 6, 0),    # low cut only (fhi at Nyquist)
    ((256, 9), 0.004, 3.0, 30.0, 5, 7, 0),       # odd poles after halving
    ((256, 9), 0.004, 3.0, 30.0, 3, 5, 1),       # odd poles, minimum phase
    ((200, 5), 0.001, 20.0, 200.0, 1, 1, 0),     # one pole
    ((120, 6, 5), 0.004, 8.0, 50.0, 4, 8, 0),    # 3-D array
    ((1000, 1), 0.004, 2.0, 80.0, 6, 6, 0),      # one trace
]


def main():
    rng = np.random.default_rng(20241206)
    das = W.das2d(n1=1000, n2=60, nev=8, seed=11)
    arrays, meta = {}, []
    for k, (shape, dt, flo, fhi, nplo, nphi, phase) in enumerate(CASES):
        if len(shape) == 2 and shape[0] <= das.shape[0] and shape[1] <= das.shape[1]:
            a = np.ascontiguousarray(das[: shape[0], : shape[1]], dtype=np.float32)
        else:
            a = rng.standard_normal(shape).astype(np.float32)
        n1 = shape[0]
        n2 = shape[1] if len(shape) > 1 else 1
        n3 = shape[2] if len(shape) > 2 else 1
        out = bpcfun.cbp(a.flatten(order="F"), n1, n2, n3, dt, flo, fhi, nplo, nphi, phase, 0)
        arrays[f"in_{k}"] = a
        arrays[f"out_{k}"] = np.asarray(out, dtype=np.float32).reshape(shape, order="F")
        meta.append({"k": k, "shape": list(shape), "dt": dt, "flo": flo, "fhi": fhi,
                     "nplo": nplo, "nphi": nphi, "phase": phase})
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    path = os.path.join(HERE, "golden_bp.npz")
    np.savez_compressed(path, **arrays)
    print(f"wrote {path}: {len(meta)} cases")


if __name__ == "__main__":
    main()
