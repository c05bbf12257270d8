"""The painting kernel's per-thread code (pwd_paint.cuh) run on the CPU for
both threads of a section (tests/emu/paint_emu.cpp) against the reference's
own outputs (golden_paint.npz) and the oracle, bit for bit.  The GPU runs the
same code in tests/test_gpu_zpaint.py."""
import ctypes
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "golden_paint.npz")


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("paint_emu") / "libpaint_emu.so")
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-std=c++17", "-o", so,
                    os.path.join(HERE, "emu", "paint_emu.cpp")], check=True)
    lib = ctypes.CDLL(so)
    P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    lib.emu_paint2d.argtypes = [P, P, P, I, I, I, I, F]
    lib.emu_paint2d.restype = I

    def run(dip, seed, order, i0, eps):
        n1, n2 = dip.shape
        d = np.ascontiguousarray(np.asarray(dip, np.float32).reshape(-1, order="F"))
        s = np.ascontiguousarray(seed, np.float32).reshape(-1)
        out = np.full(n1 * n2, 7.0, np.float32)
        p = lambda a: a.ctypes.data_as(P)  # noqa: E731
        assert lib.emu_paint2d(p(d), p(s), p(out), n1, n2, order, i0, eps) == 0
        return out.reshape(n1, n2, order="F")

    return run


def test_emulated_kernel_matches_reference(emu):
    z = np.load(GOLDEN)
    for m in json.loads(bytes(z["meta"]).decode()):
        k = m["k"]
        got = emu(z[f"dip_{k}"], z[f"seed_{k}"], m["order"], m["i0"], m["eps"])
        assert np.array_equal(got, z[f"out_{k}"]), k


CASES = [
    # n1, n2, order, i0, eps, seed
    (120, 40, 1, 0, 0.01, 1),
    (120, 40, 2, 39, 0.1, 2),
    (97, 33, 3, 16, 0.05, 3),
    (64, 20, 4, 7, 0.01, 4),
    (4, 6, 2, 3, 0.1, 5),       # shortest trace
    (50, 1, 2, 0, 0.1, 6),      # one trace: the seed alone
]


@pytest.mark.parametrize("case", CASES, ids=[f"paint-{c[0]}x{c[1]}-o{c[2]}-i{c[3]}"
                                             for c in CASES])
def test_emulated_kernel_matches_oracle(emu, case):
    n1, n2, order, i0, eps, seed = case
    rng = np.random.default_rng(seed)
    dip = (rng.standard_normal((n1, n2)) * 1.5).astype(np.float32)
    tr = np.linspace(0.0, 0.004 * (n1 - 1), n1).astype(np.float32) + rng.standard_normal(
        n1).astype(np.float32) * 0.01
    want = O.paint2d(dip, tr, order=order, i0=i0, eps=eps)
    got = emu(dip, tr, order, i0, eps)
    assert np.array_equal(got, want)


def test_emulated_stacked_sections_match_oracle(tmp_path):
    """The batch decomposition over 4 stacked sections (threads run in
    reverse order) gives each section's oracle painting."""
    so = str(tmp_path / "libpaint_emu.so")
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-std=c++17", "-o", so,
                    os.path.join(HERE, "emu", "paint_emu.cpp")], check=True)
    lib = ctypes.CDLL(so)
    P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    lib.emu_paint2d_batch.argtypes = [P, P, P, I, I, I, I, I, F]
    rng = np.random.default_rng(30)
    n1, n2, nsec, i0 = 60, 17, 4, 5
    dips = [(rng.standard_normal((n1, n2)) * 1.2).astype(np.float32) for _ in range(nsec)]
    seeds = [rng.standard_normal(n1).astype(np.float32) for _ in range(nsec)]
    d = np.ascontiguousarray(np.concatenate([p.reshape(-1, order="F") for p in dips]))
    s = np.ascontiguousarray(np.concatenate(seeds))
    out = np.full(nsec * n1 * n2, 7.0, np.float32)
    p = lambda a: a.ctypes.data_as(P)  # noqa: E731
    assert lib.emu_paint2d_batch(p(d), p(s), p(out), n1, n2, nsec, 2, i0, 0.1) == 0
    for k in range(nsec):
        want = O.paint2d(dips[k], seeds[k], order=2, i0=i0, eps=0.1).reshape(-1, order="F")
        assert np.array_equal(out[k * n1 * n2:(k + 1) * n1 * n2], want), k
