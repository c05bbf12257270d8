"""The sparse-data interpolation's CG driver and per-sample kernel code
(pwd_sint.cuh) run on the CPU with the oracle's smoothing in place of the GPU
spray kernels (tests/emu/sint_emu.cpp), against the reference's own outputs
(golden_sint.npz) and the oracle: bit for bit.  The GPU runs the same driver
with its kernels in tests/test_gpu_zsint.py."""
import ctypes
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "golden_sint.npz")
Z = np.load(GOLDEN)
META = [m for m in json.loads(bytes(Z["meta"]).decode()) if m["dim"] == 2]


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("sint_emu") / "libsint_emu.so")
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-std=c++17", "-o", so,
                    os.path.join(HERE, "emu", "sint_emu.cpp")], check=True)
    lib = ctypes.CDLL(so)
    P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    lib.emu_sint2d.argtypes = [P, P, P, P, I, I, I, I, I, F]
    lib.emu_sint2d.restype = I

    def run(d, mask, dip, niter, eps, ns, order):
        n1, n2 = d.shape
        fl = lambda a: np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1, order="F"))  # noqa: E731
        dd, mm, pp = fl(d), fl(mask), fl(dip)
        out = np.full_like(dd, 7.0)
        p = lambda a: a.ctypes.data_as(P)  # noqa: E731
        assert lib.emu_sint2d(p(dd), p(pp), p(mm), p(out), n1, n2, niter, ns, order, eps) == 0
        return out.reshape(n1, n2, order="F")

    return run


@pytest.mark.parametrize("m", META, ids=[f"sint2d-{m['k']}" for m in META])
def test_driver_matches_reference(emu, m):
    k = m["k"]
    got = emu(Z[f"d2_{k}"], Z[f"m2_{k}"], Z[f"p2_{k}"], m["niter"], m["eps"], m["ns"], m["order"])
    assert np.array_equal(got, Z[f"o2_{k}"])


CASES = [
    # n1, n2, niter, ns, order, eps, known fraction, seed
    (120, 40, 25, 2, 2, 0.01, 0.3, 1),
    (64, 30, 40, 1, 4, 0.05, 0.5, 2),
    (50, 12, 5, 0, 1, 0.01, 0.2, 3),     # no spray: S is the identity
    (40, 10, 10, 2, 2, 0.01, 1.0, 4),    # everything known
    (40, 10, 10, 2, 2, 0.01, 0.0, 5),    # nothing known: r0 = 0, returns S d
    (40, 10, 0, 1, 1, 0.01, 0.4, 6),     # no iterations
    (16, 4, 30, 0, 1, 0.01, 0.5, 2),     # the stopping test ends the loop after one step
]


@pytest.mark.parametrize("case", CASES, ids=[f"sint2d-{c[0]}x{c[1]}-it{c[2]}-ns{c[3]}-o{c[4]}"
                                             for c in CASES])
def test_driver_matches_oracle(emu, case):
    n1, n2, niter, ns, order, eps, frac, seed = case
    rng = np.random.default_rng(seed)
    keep = (rng.random(n2) < frac).astype(np.float32)
    mask = np.repeat(keep[None, :], n1, 0)
    d = (rng.standard_normal((n1, n2)) * mask).astype(np.float32)
    dip = (rng.standard_normal((n1, n2)) * 0.7).astype(np.float32)
    want = O.sint2d(d, mask, dip, niter=niter, eps=eps, ns=ns, order=order)
    got = emu(d, mask, dip, niter, eps, ns, order)
    assert np.array_equal(got, want)


META3 = [m for m in json.loads(bytes(Z["meta"]).decode()) if m["dim"] == 3]


@pytest.fixture(scope="module")
def emu3(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("sint3_emu") / "libsint_emu.so")
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-std=c++17", "-o", so,
                    os.path.join(HERE, "emu", "sint_emu.cpp")], check=True)
    lib = ctypes.CDLL(so)
    P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    lib.emu_sint3d.argtypes = [P, P, P, P, P, I, I, I, I, I, I, I, I, F]
    lib.emu_sint3d.restype = I

    def run(d, mask, pi, px, niter, eps, ns, order):
        n1, n2, n3 = d.shape
        fl = lambda a: np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1, order="F"))  # noqa: E731
        dd, mm, pp, qq = fl(d), fl(mask), fl(pi), fl(px)
        out = np.full_like(dd, 7.0)
        p = lambda a: a.ctypes.data_as(P)  # noqa: E731
        assert lib.emu_sint3d(p(dd), p(pp), p(qq), p(mm), p(out), n1, n2, n3, niter, ns[0],
                              ns[1], order[0], order[1], eps) == 0
        return out.reshape(n1, n2, n3, order="F")

    return run


@pytest.mark.parametrize("m", META3, ids=[f"sint3d-{m['k']}" for m in META3])
def test_driver_3d_matches_reference(emu3, m):
    k = m["k"]
    got = emu3(Z[f"d3_{k}"], Z[f"m3_{k}"], Z[f"pi3_{k}"], Z[f"px3_{k}"], m["niter"], m["eps"],
               m["ns"], m["order"])
    assert np.array_equal(got, Z[f"o3_{k}"])


CASES3 = [
    # n1, n2, n3, niter, (ns1, ns2), (order1, order2), eps, known fraction, seed
    (40, 9, 7, 8, (1, 2), (2, 1), 0.01, 0.3, 1),
    (24, 5, 11, 12, (2, 1), (1, 3), 0.05, 0.5, 2),
    (16, 6, 1, 6, (1, 1), (2, 2), 0.01, 0.4, 3),   # one slice
    (16, 6, 1, 6, (2, 2), (2, 2), 0.01, 0.4, 5),   # one slice, crossline weight 3 (rounds)
    (16, 1, 6, 6, (1, 1), (2, 2), 0.01, 0.4, 4),   # one inline trace
]


@pytest.mark.parametrize("case", CASES3, ids=[f"sint3d-{c[0]}x{c[1]}x{c[2]}-it{c[3]}"
                                              for c in CASES3])
def test_driver_3d_matches_oracle(emu3, case):
    n1, n2, n3, niter, ns, order, eps, frac, seed = case
    rng = np.random.default_rng(seed)
    keep = (rng.random((n2, n3)) < frac).astype(np.float32)
    mask = np.repeat(keep[None], n1, 0)
    d = (rng.standard_normal((n1, n2, n3)) * mask).astype(np.float32)
    pi = (rng.standard_normal((n1, n2, n3)) * 0.6).astype(np.float32)
    px = (rng.standard_normal((n1, n2, n3)) * 0.6).astype(np.float32)
    want = O.sint3d(d, mask, pi, px, niter=niter, eps=eps, ns1=ns[0], ns2=ns[1], order1=order[0],
                    order2=order[1])
    got = emu3(d, mask, pi, px, niter, eps, ns, order)
    assert np.array_equal(got, want)
