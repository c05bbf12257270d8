"""FP64 fixture of the batched 3-D interpolation workload (64 patches of
``workloads.patches3d(seed=2023)``: dip3d niter=5, liter=10, order=2,
rect=5,5,5 on each full patch, then soint3d order=2, niter=20 of the patch
with half its traces masked).

For every patch the oracle's double instantiation runs the whole chain (the
reference algorithm evaluated in double); the fixture keeps the
interpolated values at 2048 seeded random samples of the masked traces (as
float32), the sample indices, and per patch over all masked samples: the
reference FP32 chain's (the float oracle, bit-exact with the reference)
relative L2 distance to the FP64 chain, and the FP64 chain's relative L2
distance to the true (unmasked) data.

    python tests/golden/make_golden_patches.py [workers]

Takes a few minutes on 8 cores.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

NPER = 2048
SEED = 2023


def _chain(O, d, m, precision):
    pi, px = O.dip3d(d, 5, 10, 2, (5, 5, 5), precision=precision)
    return O.soint3d(d * m, m, pi, px, order=2, niter=20, precision=precision)


def _one(args):
    k, d, m = args
    from oracle import oracle as O

    f64 = np.asarray(_chain(O, d, m, "f64"), np.float64).reshape(-1, order="F")
    f32 = np.asarray(_chain(O, d, m, "f32"), np.float64).reshape(-1, order="F")
    truth = np.asarray(d, np.float64).reshape(-1, order="F")
    hole = np.flatnonzero(m.reshape(-1, order="F") == 0)
    rng = np.random.default_rng(3000 + k)
    idx = np.sort(rng.choice(hole, min(NPER, hole.size), replace=False)).astype(np.int64)

    def rel(a, b):
        den = np.linalg.norm(b)
        return float(np.linalg.norm(a - b) / den) if den > 0 else 0.0

    return (k, idx, f64[idx], rel(f32[hole], f64[hole]), rel(f64[hole], truth[hole]))


def main():
    import workloads as W

    workers = int(sys.argv[1]) if len(sys.argv) > 1 else max(1, (os.cpu_count() or 2) - 1)
    pairs = W.patches3d(seed=SEED, count=64)
    res = [None] * len(pairs)
    with mp.get_context("spawn").Pool(workers) as pool:
        for r in pool.imap_unordered(_one, [(k, d, m) for k, (d, m) in enumerate(pairs)]):
            res[r[0]] = r
    np.savez_compressed(
        os.path.join(HERE, "golden_patches_f64.npz"),
        shapes=np.array([d.shape for d, _ in pairs], np.int64),
        count=np.array([len(r[1]) for r in res], np.int64),
        idx=np.concatenate([r[1] for r in res]),
        interp64=np.concatenate([r[2] for r in res]).astype(np.float32),
        ref32_rel_l2_vs_f64=np.array([r[3] for r in res], np.float64),
        f64_rel_l2_vs_truth=np.array([r[4] for r in res], np.float64))
    print("reference FP32 chain vs FP64 on the masked traces, worst patch:", max(r[3] for r in res))
    print("FP64 chain vs the true data on the masked traces, median patch:",
          float(np.median([r[4] for r in res])))


if __name__ == "__main__":
    main()
