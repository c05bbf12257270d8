"""FP64 fixture of the batched workload (512 sections of
``workloads.batch2d(seed=2023)``; dip2d niter=5, liter=10, order=2,
rect=10,10,1, then somean2d ns=6, order=2, eps=0.01).

For every section the oracle's double instantiation gives the FP64 slopes
and the FP64 structure-oriented mean of the section on those slopes (the
reference algorithm evaluated in double); the fixture keeps both at 512
seeded random samples of each section (as float32: the fields' rounding to
float32, 6e-8 relative, is far below the 1e-4 bar they are used for), plus
each section's sample indices and the reference FP32 slopes' (the float
oracle, bit-exact with the reference) relative L2 distance to FP64 over the
whole section.

    python tests/golden/make_golden_batch.py [workers]

Takes about ten minutes on 8 cores.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

NPER = 512
SEED = 2023


def _one(args):
    k, s = args
    from oracle import oracle as O

    f64 = O.dip2d(s, 5, 10, 2, (10, 10, 1), precision="f64")
    f32 = O.dip2d(s, 5, 10, 2, (10, 10, 1))
    mean = O.somean2d(s, f64, 6, 2, 0.01, 0, "f64")
    rng = np.random.default_rng(1000 + k)
    idx = np.sort(rng.choice(s.size, min(NPER, s.size), replace=False)).astype(np.int64)
    flat = lambda a: np.asarray(a, np.float64).reshape(-1, order="F")  # noqa: E731
    den = np.linalg.norm(flat(f64))
    rel = float(np.linalg.norm(flat(f32) - flat(f64)) / den) if den > 0 else 0.0
    return k, idx, flat(f64)[idx], flat(mean)[idx], rel


def main():
    import workloads as W

    workers = int(sys.argv[1]) if len(sys.argv) > 1 else max(1, (os.cpu_count() or 2) - 1)
    secs = W.batch2d(seed=SEED, count=512)
    res = [None] * len(secs)
    with mp.get_context("spawn").Pool(workers) as pool:
        for r in pool.imap_unordered(_one, list(enumerate(secs))):
            res[r[0]] = r
    cnt = np.array([len(r[1]) for r in res], np.int64)
    np.savez_compressed(
        os.path.join(HERE, "golden_batch_f64.npz"),
        shapes=np.array([s.shape for s in secs], np.int64), count=cnt,
        idx=np.concatenate([r[1] for r in res]),
        dip64=np.concatenate([r[2] for r in res]).astype(np.float32),
        mean64=np.concatenate([r[3] for r in res]).astype(np.float32),
        ref32_rel_l2_vs_f64=np.array([r[4] for r in res], np.float64))
    print("reference FP32 vs FP64, worst section:", max(r[4] for r in res))


if __name__ == "__main__":
    main()
