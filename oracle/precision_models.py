"""Half-precision storage measured with the oracle's precision models (test
infrastructure: prints the table of storage choices and their error).

  python oracle/precision_models.py

Two storage choices of the throughput path are modelled in the float
restatement of the reference, everything else unchanged:
  - the spray's factor store (the taps the filter application reads and the
    LDL' factors the solves read: 15 floats a sample) in FP16 or BF16
    (orc_set_store16), against the structure-oriented mean (ns 6) and median
    (ns 10) of the FP64 evaluation given the same FP64 slopes;
  - the shaping CG's conjugate directions (sp, sx, sr) in FP16 or BF16
    (orc_set_cg_store16), with the smoothing exact (TRI_EXACT, as the mixed
    mode's convolution), against the FP64 slopes.
Sections of the 512-section workload (workloads.batch2d(seed=2023)) and a
600 x 200 DAS piece.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# run as a script, this folder is first on the path and its oracle.py would
# shadow the oracle package
sys.path[:] = [p for p in sys.path if os.path.abspath(p or ".") != HERE]
sys.path.insert(0, os.path.dirname(HERE))

import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402


def rel(a, b):
    return float(np.linalg.norm(np.float64(a) - b) / np.linalg.norm(b))


def main():
    lib = ctypes.CDLL(O._LIB_PATH)
    names = {0: "FP32", 1: "FP16", 2: "BF16"}
    secs = W.batch2d(seed=2023, count=512)
    # factor store
    pick = [secs[k][:, :min(secs[k].shape[1], 120)].copy() for k in (0, 1, 2, 66, 256, 300)]
    mean = {m: [] for m in names}
    for s in pick:
        lib.orc_set_store16(0)
        p64 = O.dip2d(s, 5, 10, 2, (10, 10, 1), precision="f64")
        m64 = O.somean2d(s, p64, 6, 2, 0.01, 0, "f64")
        for m in names:
            lib.orc_set_store16(m)
            mean[m].append(rel(O.somean2d(s, p64.astype(np.float32), 6, 2, 0.01), m64))
    lib.orc_set_store16(0)
    das = W.das2d(n1=600, n2=200, nev=8)
    p64 = O.dip2d(das, 5, 20, 2, (10, 10, 1), precision="f64")
    f64 = O.somf2d(das, p64, 10, 2, 0.01, precision="f64")
    med = {}
    for m in names:
        lib.orc_set_store16(m)
        med[m] = rel(O.somf2d(das, p64.astype(np.float32), 10, 2, 0.01), f64)
    lib.orc_set_store16(0)
    for m in names:
        print(f"spray factor store {names[m]}: somean2d(ns 6) vs FP64 max {max(mean[m]):.2e}, "
              f"median {np.median(mean[m]):.2e}; somf2d(ns 10) {med[m]:.2e}")
    # CG directions
    res = {m: [] for m in names}
    for k in (0, 1, 2, 3, 300, 410):
        s = secs[k]
        lib.orc_set_cg_store16(0)
        f64 = O.dip2d(s, 5, 10, 2, (10, 10, 1), precision="f64")
        for m in names:
            lib.orc_set_cg_store16(m)
            res[m].append(rel(O.dip2d(s, 5, 10, 2, (10, 10, 1), flags=O.TRI_EXACT), f64))
    lib.orc_set_cg_store16(0)
    for m in names:
        print(f"CG directions {names[m]}: slopes vs FP64 max {max(res[m]):.2e}, "
              f"median {np.median(res[m]):.2e}")


if __name__ == "__main__":
    main()
