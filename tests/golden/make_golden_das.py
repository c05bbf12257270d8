"""Full-size golden fixture of the DAS slope workload (2000 x 5000 record,
dip2d niter=5, liter=20, order=2, rect=10,10,1).

Runs the reference's own FP32 dipc (oracle/_ref/dipcfun, compiled from the
reference sources by ``make -C oracle ref``), the FP64 evaluation of the
same algorithm (the oracle's double instantiation) and the oracle's FP32
restatement with its dot products and residual energies summed in the GPU
plain path's order (flag GPU_DOTS; everything else is the reference's
float arithmetic) on the seeded record of ``workloads.das2d(seed=2023)``,
and stores the three slope fields at 32768 seeded random samples, plus
their relative L2 distances to each other over the whole record.

    make -C oracle ref && python tests/golden/make_golden_das.py

Takes a few minutes on one core.  The fixture is what the full-size GPU
tests read.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
sys.path.insert(0, ROOT)

import dipcfun  # noqa: E402

import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

NSAMPLE = 32768


def main():
    d = W.das2d(seed=2023)
    n1, n2 = d.shape
    fd = os.dup(1)
    nul = os.open(os.devnull, os.O_WRONLY)
    os.dup2(nul, 1)
    try:
        # dipc positional tuple (dip_cfuns.c:1708) as dip2dc passes it
        ref = np.asarray(dipcfun.dipc(np.float32(d.flatten(order="F")), n1, n2, 1, 5, 20, 2,
                                      0.01, 1.0, 1e-6, 10, 10, 1, 0, 0), np.float32)
    finally:
        os.dup2(fd, 1)
        os.close(fd)
        os.close(nul)
    ref = ref.reshape(n1, n2, order="F")
    f64 = O.dip2d(d, 5, 20, 2, (10, 10, 1), precision="f64")
    gpuo = O.dip2d(d, 5, 20, 2, (10, 10, 1), flags=O.GPU_DOTS)
    rng = np.random.default_rng(7)
    idx = np.sort(rng.choice(d.size, NSAMPLE, replace=False)).astype(np.int64)
    flat = lambda a: np.asarray(a).reshape(-1, order="F")  # noqa: E731
    def rel_l2(a, b):
        a, b = np.float64(flat(a)), np.float64(flat(b))
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    rel = rel_l2(ref, f64)
    np.savez_compressed(os.path.join(HERE, "golden_das_full.npz"), idx=idx,
                        ref32=flat(ref)[idx].astype(np.float32),
                        f64=flat(f64)[idx].astype(np.float64),
                        gpuorder32=flat(gpuo)[idx].astype(np.float32),
                        ref32_rel_l2_vs_f64=np.float64(rel),
                        gpuorder32_rel_l2_vs_ref32=np.float64(rel_l2(gpuo, ref)),
                        gpuorder32_rel_l2_vs_f64=np.float64(rel_l2(gpuo, f64)),
                        shape=np.array([n1, n2]))
    print("reference FP32 vs FP64 relative L2 over the record:", rel)
    print("GPU-order FP32 vs reference FP32:", rel_l2(gpuo, ref), " vs FP64:", rel_l2(gpuo, f64))


if __name__ == "__main__":
    main()
