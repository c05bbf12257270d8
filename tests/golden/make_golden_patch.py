"""Golden fixtures of pyseistr's patching, made by the reference itself.

Loads the reference's pure-numpy module pyseistr/patch.py on its own (the
package's __init__ needs matplotlib) and runs patch2d / patch3d and their
inverses on small seeded arrays, storing inputs, parameters and outputs in
tests/golden/golden_patch.npz.  The reference is only present where the
fixtures are made; the committed file is what the tests read.

    python tests/golden/make_golden_patch.py [path to the reference's patch.py]

Cases cover padding on none, some and all axes, windows longer than an axis,
strides larger than the window (uncovered samples: NaN in the inverse), and
the six padding patterns of patch3d_inv that the reference handles (its two
others, padding axes 1 and 3 but not 2 or axes 2 and 3 but not 1, leave its
output array unassigned and raise).
"""
from __future__ import annotations

import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT = os.path.join(os.sep, "root", "reference", "pyseistr", "patch.py")


def load(path):
    spec = importlib.util.spec_from_file_location("ref_patch", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


CASES_2D = [  # (n1, n2, l1, l2, s1, s2)
    (32, 24, 8, 8, 4, 4),     # no padding
    (37, 29, 8, 8, 4, 4),     # both axes padded
    (40, 29, 16, 8, 8, 4),    # axis 2 padded
    (5, 30, 8, 6, 4, 3),      # window longer than axis 1
    (30, 22, 4, 4, 6, 5),     # stride larger than the window
    (64, 50, 16, 16, 16, 16),  # no overlap
]
CASES_3D = [  # (n1, n2, n3, l1, l2, l3, s1, s2, s3)
    (12, 10, 8, 4, 4, 4, 2, 2, 2),   # no padding
    (13, 11, 9, 4, 4, 4, 2, 2, 2),   # all padded
    (13, 11, 8, 4, 4, 4, 2, 2, 2),   # axes 1, 2
    (13, 10, 8, 4, 4, 4, 2, 2, 2),   # axis 1
    (12, 11, 8, 4, 4, 4, 2, 2, 2),   # axis 2
    (12, 10, 9, 4, 4, 4, 2, 2, 2),   # axis 3
    (20, 9, 7, 8, 4, 3, 4, 3, 2),    # uneven windows
]


def main():
    ref = load(sys.argv[1] if len(sys.argv) > 1 else DEFAULT)
    rng = np.random.default_rng(20241205)
    arrays, meta = {}, []
    for k, (n1, n2, l1, l2, s1, s2) in enumerate(CASES_2D):
        a = rng.standard_normal((n1, n2)).astype(np.float32)
        x = ref.patch2d(a, l1, l2, s1, s2)
        b = ref.patch2d_inv(x, n1, n2, l1, l2, s1, s2)
        arrays[f"a2_{k}"], arrays[f"x2_{k}"], arrays[f"b2_{k}"] = a, np.asarray(x), np.asarray(b)
        meta.append({"dim": 2, "k": k, "n": [n1, n2], "l": [l1, l2], "s": [s1, s2]})
    for k, (n1, n2, n3, l1, l2, l3, s1, s2, s3) in enumerate(CASES_3D):
        a = rng.standard_normal((n1, n2, n3)).astype(np.float32)
        x = ref.patch3d(a, l1, l2, l3, s1, s2, s3)
        b = ref.patch3d_inv(np.asarray(x)[:, :, 0], n1, n2, n3, l1, l2, l3, s1, s2, s3)
        arrays[f"a3_{k}"], arrays[f"x3_{k}"], arrays[f"b3_{k}"] = a, np.asarray(x), np.asarray(b)
        meta.append({"dim": 3, "k": k, "n": [n1, n2, n3], "l": [l1, l2, l3],
                     "s": [s1, s2, s3]})
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    out = os.path.join(HERE, "golden_patch.npz")
    np.savez_compressed(out, **arrays)
    print(f"wrote {out}: {len(meta)} cases")


if __name__ == "__main__":
    main()
