"""Generate the golden fixtures from the reference implementation itself.

Runs pyseistr's own C extensions (dipcfun, sofcfun, sof3dcfun, soint3dcfun),
compiled from the reference sources by ``make -C oracle ref`` into
``oracle/_ref/``, on small seeded inputs and stores inputs and outputs as
float32 in ``tests/golden/*.npz``.  The reference is only present where the
fixtures are made; the committed fixtures are what the tests read.

    make -C oracle ref && python tests/golden/make_golden.py

The call signatures are those of the reference's Python wrappers
(dip2d.py:115 dip2dc, dip3d.py:59 dip3dc, somean2d.py:36, somf2d.py:60,
somean3d.py:36, somf3d.py:54, soint3d.py:65).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref"))
sys.path.insert(0, ROOT)

import dipcfun  # noqa: E402
import sof3dcfun  # noqa: E402
import sofcfun  # noqa: E402
import soint3dcfun  # noqa: E402

import workloads as W  # noqa: E402


def _quiet(fn, *args):
    """Run a reference call with its C-level stdout silenced."""
    sys.stdout.flush()
    fd = os.dup(1)
    nul = os.open(os.devnull, os.O_WRONLY)
    os.dup2(nul, 1)
    try:
        return fn(*args)
    finally:
        os.dup2(fd, 1)
        os.close(fd)
        os.close(nul)


def F(a):
    return np.float32(a).flatten(order="F")


def ref_dip(d, niter, liter, order, rect, mask=None):
    sh = d.shape
    n1, n2 = sh[0], sh[1]
    n3 = sh[2] if d.ndim == 3 else 1
    if mask is None:
        din, hasmask = F(d), 0
    else:
        din, hasmask = np.concatenate([F(d), F(mask)]), 1
    return _quiet(dipcfun.dipc, din, n1, n2, n3, niter, liter, order, 0.01, 1.0, 1e-6,
                  rect[0], rect[1], rect[2], hasmask, 0)


def ref_somean2d(d, p, ns, order, eps, adj=0):
    n1, n2 = d.shape[0], d.shape[1]
    n3 = d.shape[2] if d.ndim == 3 else 1
    return _quiet(sofcfun.csomean2d, F(d), F(p), n1, n2, n3, ns, order, adj, eps, 0)


def ref_somf2d(d, p, ns, order, eps, option=1, nmf=None):
    n1, n2 = d.shape[0], d.shape[1]
    n3 = d.shape[2] if d.ndim == 3 else 1
    nmf = 2 * ns + 1 if nmf is None else nmf
    return _quiet(sofcfun.csomf2d, F(d), F(p), n1, n2, n3, ns, nmf, option, order, eps, 0)


def ref_somean3d(d, pi, px, r1, r2, order):
    n1, n2, n3 = d.shape
    return _quiet(sof3dcfun.csomean3d, F(d), F(pi), F(px), n1, n2, n3, r1, r2, order, 0.01, 0)


def ref_somf3d(d, pi, px, r1, r2, order, option=1, nmf=None):
    n1, n2, n3 = d.shape
    nmf = 2 * r1 * r2 + 1 if nmf is None else nmf
    return _quiet(sof3dcfun.csomf3d, F(d), F(pi), F(px), n1, n2, n3, r1, r2, nmf, option, order,
                  0.01, 0)


def ref_soint3d(d, mask, pi, px, order, niter, drift=0, seed=202223, hasmask=1, var=0.0):
    n1, n2, n3 = d.shape
    return _quiet(soint3dcfun.csoint3d, F(d), F(mask), F(pi), F(px), n1, n2, n3, order, 1, 1,
                  niter, drift, seed, hasmask, var, 0)


class Store:
    def __init__(self):
        self.arrays = {}
        self.cases = []
        self.seen = {}

    def add(self, fn, params, **arrays):
        k = len(self.cases)
        names = {}
        for name, a in arrays.items():
            a = np.asarray(a, dtype=np.float32)
            sig = (a.shape, hashlib.sha1(a.tobytes(order="F")).hexdigest())
            if sig not in self.seen:     # shared inputs are stored once
                self.seen[sig] = f"c{k}_{name}"
                self.arrays[self.seen[sig]] = a
            names[name] = self.seen[sig]
        self.cases.append({"fn": fn, "params": params, "arrays": names})

    def save(self, path):
        np.savez_compressed(path, meta=np.frombuffer(json.dumps(self.cases).encode(), np.uint8),
                            **self.arrays)
        print(f"{path}: {len(self.cases)} cases, {os.path.getsize(path) / 1e6:.2f} MB")


def tiny2d(rng, n1, n2):
    t = np.arange(n1)[:, None]
    x = np.arange(n2)[None, :]
    d = np.sin(0.7 * t - 0.9 * x) + 0.3 * rng.standard_normal((n1, n2))
    return d.astype(np.float32)


def main():
    rng = np.random.default_rng(20231203)
    S = Store()

    # --- configuration 1: the reference's CPU-runnable case, full size ----------
    d = W.plain2d()
    p = ref_dip(d, 5, 10, 2, (10, 10, 1)).reshape(d.shape, order="F")
    S.add("dip", dict(niter=5, liter=10, order=2, rect=[10, 10, 1]), d=d, out=p)
    for ns, adj in ((8, 0), (8, 1)):
        S.add("somean2d", dict(ns=ns, order=2, eps=0.01, adj=adj), d=d, p=p,
              out=ref_somean2d(d, p, ns, 2, 0.01, adj).reshape(d.shape, order="F"))
    for opt in (1, 2):
        S.add("somf2d", dict(ns=8, order=2, eps=0.01, option=opt, nmf=17), d=d, p=p,
              out=ref_somf2d(d, p, 8, 2, 0.01, opt).reshape(d.shape, order="F"))

    # --- dip2d variants: mask, order 1 and 3, rect larger than the section ------
    dm = d[:200, :40].copy()
    mask = np.ones_like(dm)
    mask[:, 7] = 0.0
    mask[50:60, 20:23] = 0.0
    S.add("dip", dict(niter=3, liter=8, order=2, rect=[6, 4, 1], mask=True), d=dm, mask=mask,
          out=ref_dip(dm, 3, 8, 2, (6, 4, 1), mask).reshape(dm.shape, order="F"))
    for order in (1, 3):
        S.add("dip", dict(niter=3, liter=6, order=order, rect=[5, 3, 1]), d=dm,
              out=ref_dip(dm, 3, 6, order, (5, 3, 1)).reshape(dm.shape, order="F"))
    small = tiny2d(rng, 24, 5)
    S.add("dip", dict(niter=2, liter=5, order=2, rect=[30, 12, 1]), d=small,
          out=ref_dip(small, 2, 5, 2, (30, 12, 1)).reshape(small.shape, order="F"))

    # --- 2-D spray filters: small and ragged edge cases ---------------------------
    for (n1, n2, ns, order) in ((9, 1, 1, 1), (12, 3, 2, 2), (7, 4, 3, 1), (40, 9, 3, 2),
                                (33, 17, 5, 3), (64, 30, 4, 2)):
        dd = tiny2d(rng, n1, n2)
        pp = (1.5 * rng.standard_normal((n1, n2))).astype(np.float32)
        for adj in (0, 1):
            S.add("somean2d", dict(ns=ns, order=order, eps=0.01, adj=adj), d=dd, p=pp,
                  out=ref_somean2d(dd, pp, ns, order, 0.01, adj).reshape(dd.shape, order="F"))
        S.add("somf2d", dict(ns=ns, order=order, eps=0.01, option=1, nmf=2 * ns + 1), d=dd, p=pp,
              out=ref_somf2d(dd, pp, ns, order, 0.01, 1).reshape(dd.shape, order="F"))
        if 2 * ns + 1 >= 5:
            S.add("somf2d", dict(ns=ns, order=order, eps=0.01, option=2, nmf=2 * ns + 1), d=dd,
                  p=pp, out=ref_somf2d(dd, pp, ns, order, 0.01, 2).reshape(dd.shape, order="F"))
    # a window longer than the spray (edge replication), dead (zero) traces,
    # and several slices (n3 > 1) handled slice by slice
    dd = tiny2d(rng, 30, 12)
    dd[:, 4] = 0.0
    pp = (rng.uniform(-2, 2, (30, 12))).astype(np.float32)
    S.add("somf2d", dict(ns=2, order=2, eps=0.05, option=1, nmf=9), d=dd, p=pp,
          out=ref_somf2d(dd, pp, 2, 2, 0.05, 1, 9).reshape(dd.shape, order="F"))
    d3 = np.stack([tiny2d(rng, 20, 6) for _ in range(3)], axis=2)
    p3 = (rng.uniform(-1, 1, d3.shape)).astype(np.float32)
    S.add("somean2d", dict(ns=2, order=2, eps=0.01, adj=0), d=d3, p=p3,
          out=ref_somean2d(d3, p3, 2, 2, 0.01).reshape(d3.shape, order="F"))
    S.add("somf2d", dict(ns=2, order=2, eps=0.01, option=1, nmf=5), d=d3, p=p3,
          out=ref_somf2d(d3, p3, 2, 2, 0.01, 1).reshape(d3.shape, order="F"))
    S.save(os.path.join(HERE, "golden_2d.npz"))

    # --- 3-D: dip3d, somean3d, somf3d, soint3d on a cut of configuration 2 -------
    S = Store()
    c = W.plain3d()[60:124, 10:34, 12:32].copy()   # 64 x 24 x 20
    pq = ref_dip(c, 5, 10, 2, (5, 5, 5))
    pi = pq[: c.size].reshape(c.shape, order="F")
    px = pq[c.size:].reshape(c.shape, order="F")
    S.add("dip", dict(niter=5, liter=10, order=2, rect=[5, 5, 5]), d=c, out_i=pi, out_x=px)
    for r1, r2 in ((2, 2), (1, 3), (0, 2)):
        S.add("somean3d", dict(r1=r1, r2=r2, order=2), d=c, pi=pi, px=px,
              out=ref_somean3d(c, pi, px, r1, r2, 2).reshape(c.shape, order="F"))
    for r1, r2, opt in ((2, 2, 1), (2, 2, 2), (1, 3, 1)):
        S.add("somf3d", dict(r1=r1, r2=r2, order=2, option=opt, nmf=2 * r1 * r2 + 1), d=c, pi=pi,
              px=px, out=ref_somf3d(c, pi, px, r1, r2, 2, opt).reshape(c.shape, order="F"))
    keep = (rng.random((c.shape[1], c.shape[2])) >= 0.5).astype(np.float32)
    mask = np.broadcast_to(keep[None], c.shape).astype(np.float32)
    din = (c * mask).astype(np.float32)
    for order, niter, drift, var in ((2, 10, 0, 0.0), (1, 6, 0, 0.0), (2, 5, 0, 0.01),
                                     (2, 5, 1, 0.0)):
        S.add("soint3d", dict(order=order, niter=niter, drift=drift, var=var, seed=202223),
              d=din, mask=mask, pi=pi, px=px,
              out=ref_soint3d(din, mask, pi, px, order, niter, drift, 202223, 1, var)
              .reshape(c.shape, order="F"))
    # tiny cube with a mask in dip3d, and a ragged cube for the spray
    t = np.random.default_rng(5).standard_normal((12, 5, 4)).astype(np.float32)
    tm = np.ones_like(t)
    tm[:, 2, 1] = 0
    pq = ref_dip(t, 2, 4, 1, (3, 2, 2), tm)
    S.add("dip", dict(niter=2, liter=4, order=1, rect=[3, 2, 2], mask=True), d=t, mask=tm,
          out_i=pq[: t.size].reshape(t.shape, order="F"), out_x=pq[t.size:].reshape(t.shape, order="F"))
    ti = (rng.uniform(-1, 1, t.shape)).astype(np.float32)
    tx = (rng.uniform(-1, 1, t.shape)).astype(np.float32)
    S.add("somean3d", dict(r1=2, r2=1, order=1), d=t, pi=ti, px=tx,
          out=ref_somean3d(t, ti, tx, 2, 1, 1).reshape(t.shape, order="F"))
    S.add("somf3d", dict(r1=2, r2=1, order=1, option=1, nmf=5), d=t, pi=ti, px=tx,
          out=ref_somf3d(t, ti, tx, 2, 1, 1, 1).reshape(t.shape, order="F"))
    S.save(os.path.join(HERE, "golden_3d.npz"))


if __name__ == "__main__":
    main()
