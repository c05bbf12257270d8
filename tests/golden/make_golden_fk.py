"""Golden fixtures of pyseistr's FK dip filter, made by the reference itself.

Loads the reference's pure-numpy module pyseistr/fk.py on its own (the
package's __init__ needs matplotlib) and runs fkdip on seeded DAS-like
sections (sizes at, below and above powers of two; cone widths as the DAS
workflow uses, demos/test_pyseistr_das.py:50), storing inputs, widths and
outputs in tests/golden/golden_fk.npz.

    python tests/golden/make_golden_fk.py [path to the reference's fk.py]
"""
from __future__ import annotations

import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DEFAULT = os.path.join(os.sep, "root", "reference", "pyseistr", "fk.py")
sys.path.insert(0, ROOT)

import workloads as W  # noqa: E402

CASES = [  # (n1, n2, w)
    (256, 128, 0.02),
    (500, 96, 0.02),
    (300, 200, 0.05),
    (129, 65, 0.005),
    (64, 1, 0.1),
]


def main():
    path = sys.argv[1] if len(sys.argv) > 1 else DEFAULT
    spec = importlib.util.spec_from_file_location("ref_fk", path)
    ref = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ref)
    arrays, meta = {}, []
    for k, (n1, n2, w) in enumerate(CASES):
        d = W.das2d(n1=n1, n2=max(n2, 2), nev=4, seed=30 + k)[:, :n2].astype(np.float32)
        arrays[f"in_{k}"] = d
        arrays[f"out_{k}"] = np.asarray(ref.fkdip(d, w))
        meta.append({"k": k, "w": w})
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    out = os.path.join(HERE, "golden_fk.npz")
    np.savez_compressed(out, **arrays)
    print(f"wrote {out}: {len(meta)} cases")


if __name__ == "__main__":
    main()
