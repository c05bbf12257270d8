"""Seeded synthetic seismic workloads for the PWD hot path.

The reference publishes no benchmark data set; these generators build the
sections and cubes of the five measured workloads from their recipes
(Ricker events of stated frequency and dip, Gaussian / spike noise, dead
channels, trace masks).  All arrays are float32 with time (n1) on axis 0,
the layout pyseistr's Python API takes.

  plain2d   501 x 100, three 25 Hz events (flat, 2 samples/trace, hyperbola
            t0=1 s v=2000 m/s dx=10 m), noise 0.2 x peak
  plain3d   201 x 60 x 60, three 30 Hz planes, dips (0,0) (1.5,-0.8) (-1,1),
            noise 0.3 x peak
  das2d     2000 x 5000, 40 linear 15-40 Hz events, slopes U[-3,3], 5 % dead
            channels, Gaussian + spike noise
  batch2d   512 sections, n1 ~ logU[256,2048], n2 ~ logU[64,1024], 1-6
            events with dips U[-4,4], SNR U[0,10] dB
  patches3d 64 cubes, n1 ~ U[128,512], n2 = n3 ~ U[32,96], planar events,
            50 % of traces masked out
"""
from __future__ import annotations

import numpy as np

DT = 0.004


def ricker(t, f):
    a = (np.pi * f * t) ** 2
    return (1.0 - 2.0 * a) * np.exp(-a)


def _add_events(d, arrivals, freqs, amps, dt=DT):
    """d[n1, ntr] += sum_e amps[e] * ricker(t - arrivals[e, tr], freqs[e]).

    arrivals are in seconds; each wavelet is evaluated on a window of +-2/f.
    """
    n1, ntr = d.shape
    tr = np.arange(ntr)
    for e in range(arrivals.shape[0]):
        f = float(freqs[e])
        half = int(np.ceil(2.0 / f / dt))
        k = np.arange(-half, half + 1)
        c = np.rint(arrivals[e] / dt).astype(np.int64)          # [ntr]
        idx = c[None, :] + k[:, None]                             # [2h+1, ntr]
        t = idx * dt - arrivals[e][None, :]
        w = (amps[e] * ricker(t, f)).astype(np.float32)
        ok = (idx >= 0) & (idx < n1)
        cols = np.broadcast_to(tr[None, :], idx.shape)
        np.add.at(d, (idx[ok], cols[ok]), w[ok])
    return d


def plain2d(seed=2023):
    """501 x 100 section with a flat, a dipping and a hyperbolic event."""
    rng = np.random.default_rng(seed)
    n1, n2, dx = 501, 100, 10.0
    x = (np.arange(n2) - n2 // 2) * dx
    arr = np.stack([
        np.full(n2, 0.4),                                   # flat
        0.3 + 2.0 * DT * np.arange(n2),                     # 2 samples / trace
        np.sqrt(1.0 + (x / 2000.0) ** 2),                   # hyperbola
    ])
    d = _add_events(np.zeros((n1, n2), np.float32), arr, [25.0] * 3, [1.0, 1.0, 1.0])
    peak = float(np.abs(d).max())
    d += (0.2 * peak * rng.standard_normal((n1, n2))).astype(np.float32)
    return d


def plain3d(seed=2023):
    """201 x 60 x 60 cube with three 30 Hz planes."""
    rng = np.random.default_rng(seed)
    n1, n2, n3 = 201, 60, 60
    i2, i3 = np.meshgrid(np.arange(n2) - n2 // 2, np.arange(n3) - n3 // 2, indexing="ij")
    i2, i3 = i2.ravel(order="F"), i3.ravel(order="F")
    planes = [(40, 0.0, 0.0), (100, 1.5, -0.8), (150, -1.0, 1.0)]
    arr = np.stack([(t0 + p * i2 + q * i3) * DT for t0, p, q in planes])
    d = _add_events(np.zeros((n1, n2 * n3), np.float32), arr, [30.0] * 3, [1.0] * 3)
    peak = float(np.abs(d).max())
    d += (0.3 * peak * rng.standard_normal(d.shape)).astype(np.float32)
    return d.reshape(n1, n2, n3, order="F")


def das2d(seed=2023, n1=2000, n2=5000, nev=40):
    """DAS-like record: linear events, dead channels, Gaussian + spike noise."""
    rng = np.random.default_rng(seed)
    x = np.arange(n2)
    slopes = rng.uniform(-3.0, 3.0, nev)
    t0 = rng.uniform(0.0, n1 * DT, nev)
    xc = rng.uniform(0, n2, nev)
    arr = (t0[:, None] + slopes[:, None] * (x[None, :] - xc[:, None]) * DT)
    freqs = rng.uniform(15.0, 40.0, nev)
    amps = rng.uniform(0.5, 1.0, nev) * rng.choice([-1.0, 1.0], nev)
    d = _add_events(np.zeros((n1, n2), np.float32), arr, freqs, amps)
    peak = float(np.abs(d).max())
    d += (0.2 * peak * rng.standard_normal((n1, n2))).astype(np.float32)
    nspike = (n1 * n2) // 2000
    si = rng.integers(0, n1, nspike)
    sj = rng.integers(0, n2, nspike)
    d[si, sj] += (rng.choice([-1.0, 1.0], nspike) * rng.uniform(2.0, 5.0, nspike) * peak).astype(np.float32)
    dead = rng.choice(n2, n2 // 20, replace=False)
    d[:, dead] = 0.0
    return d


def _section(rng, n1, n2):
    nev = int(rng.integers(1, 7))
    x = np.arange(n2)
    dips = rng.uniform(-4.0, 4.0, nev)
    t0 = rng.uniform(0.1, 0.9, nev) * n1 * DT
    arr = t0[:, None] + dips[:, None] * (x[None, :] - n2 / 2) * DT
    freqs = rng.uniform(15.0, 40.0, nev)
    d = _add_events(np.zeros((n1, n2), np.float32), arr, freqs, np.ones(nev))
    snr_db = rng.uniform(0.0, 10.0)
    ps = float(np.mean(d.astype(np.float64) ** 2)) or 1.0
    sigma = np.sqrt(ps / 10.0 ** (snr_db / 10.0))
    d += (sigma * rng.standard_normal((n1, n2))).astype(np.float32)
    return d


def batch2d_shapes(seed=2023, count=512, n1_range=(256, 2048), n2_range=(64, 1024)):
    rng = np.random.default_rng(seed)
    n1 = np.exp(rng.uniform(np.log(n1_range[0]), np.log(n1_range[1]), count)).astype(int)
    n2 = np.exp(rng.uniform(np.log(n2_range[0]), np.log(n2_range[1]), count)).astype(int)
    return list(zip(n1.tolist(), n2.tolist()))


def batch2d(seed=2023, count=512, n1_range=(256, 2048), n2_range=(64, 1024)):
    """`count` independent sections of log-uniform size."""
    shapes = batch2d_shapes(seed, count, n1_range, n2_range)
    rng = np.random.default_rng(seed + 1)
    return [_section(rng, a, b) for a, b in shapes]


def patches3d(seed=2023, count=64, n1_range=(128, 512), n23_range=(32, 96)):
    """`count` cubes with planar events and a 50 % trace mask.

    Returns a list of (full, mask) pairs; mask is 1 on kept traces.
    """
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n1 = int(rng.integers(n1_range[0], n1_range[1] + 1))
        n2 = n3 = int(rng.integers(n23_range[0], n23_range[1] + 1))
        nev = int(rng.integers(2, 5))
        i2, i3 = np.meshgrid(np.arange(n2) - n2 / 2, np.arange(n3) - n3 / 2, indexing="ij")
        i2, i3 = i2.ravel(order="F"), i3.ravel(order="F")
        t0 = rng.uniform(0.15, 0.85, nev) * n1
        p = rng.uniform(-1.5, 1.5, nev)
        q = rng.uniform(-1.5, 1.5, nev)
        arr = np.stack([(t0[e] + p[e] * i2 + q[e] * i3) * DT for e in range(nev)])
        d = _add_events(np.zeros((n1, n2 * n3), np.float32), arr,
                        rng.uniform(20.0, 35.0, nev), rng.uniform(0.5, 1.0, nev))
        d = d.reshape(n1, n2, n3, order="F")
        keep = (rng.random((n2, n3)) >= 0.5).astype(np.float32)
        mask = np.broadcast_to(keep[None], d.shape).astype(np.float32)
        out.append((d, mask))
    return out
