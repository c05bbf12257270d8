"""Loader for the golden fixtures in tests/golden/ (made by make_golden.py
from the reference's own compiled C)."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    """Yield (index, fn, params, arrays) for every case of golden_<name>.npz."""
    z = np.load(os.path.join(GOLDEN, f"golden_{name}.npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    out = []
    for k, case in enumerate(meta):
        arrays = {n: z[key] for n, key in case["arrays"].items()}
        out.append((k, case["fn"], case["params"], arrays))
    return out


def ids(cases):
    return [f"{fn}-{k}" for k, fn, _, _ in cases]
