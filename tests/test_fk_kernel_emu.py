"""The FK dip filter's per-thread code (pwd_fk.cuh: Stockham FFT passes,
transposes, cone mask) run on the CPU in the order of the GPU launches
(tests/emu/fk_emu.cpp) against the oracle and the reference's own outputs
(golden_fk.npz).  Not bit for bit (numpy's FFTs round differently): held to
1e-6 relative L2 for float32 input, whose forward FFTs run in complex64 on
both sides, and 1e-12 for float64 input.  The GPU runs the same code in
tests/test_gpu_zfk.py."""
import ctypes
import json
import os
import subprocess

import numpy as np
import pytest

from gpu_util import rel_l2
from oracle import fk_oracle as F

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "golden_fk.npz")
TOL32, TOL64 = 1e-6, 1e-12


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("fk_emu") / "libfk_emu.so")
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-std=c++17", "-o", so,
                    os.path.join(HERE, "emu", "fk_emu.cpp")], check=True)
    lib = ctypes.CDLL(so)
    P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lib.emu_fkdip.argtypes = lib.emu_fkdip_f64.argtypes = [P, P, I, I, D]

    def run(d, w):
        n1, n2 = d.shape
        x = np.ascontiguousarray(d.reshape(-1, order="F"))
        out = np.full(n1 * n2, 7.0, np.float64)
        fn = lib.emu_fkdip_f64 if d.dtype == np.float64 else lib.emu_fkdip
        assert fn(x.ctypes.data_as(P), out.ctypes.data_as(P), n1, n2, w) == 0
        return out.reshape(n1, n2, order="F")

    return run


def test_emulated_kernels_match_reference(emu):
    z = np.load(GOLDEN)
    for m in json.loads(bytes(z["meta"]).decode()):
        k = m["k"]
        d, want = z[f"in_{k}"], z[f"out_{k}"]
        got = emu(d, m["w"])
        assert got.shape == want.shape
        assert rel_l2(got, want) <= (TOL64 if d.dtype == np.float64 else TOL32), k


CASES = [
    # n1, n2, w, dtype, seed
    (100, 30, 0.05, np.float32, 1),
    (300, 97, 0.01, np.float32, 2),
    (64, 64, 0.1, np.float32, 3),
    (100, 30, 0.05, np.float64, 4),
    (1, 5, 0.2, np.float32, 5),     # one sample per trace
    (7, 1, 0.3, np.float32, 6),     # one trace
    (2, 2, 0.5, np.float64, 7),
    (257, 129, -0.03, np.float32, 8),  # negative width: the cone test as the reference's
    (64, 40, 2.0, np.float32, 9),      # a cone wider than the plane
    (3, 3, 0.5, np.float64, 10),
]


@pytest.mark.parametrize("case", CASES, ids=[f"fk-{c[0]}x{c[1]}-w{c[2]}-{np.dtype(c[3]).name}"
                                             for c in CASES])
def test_emulated_kernels_match_oracle(emu, case):
    n1, n2, w, dt, seed = case
    d = np.random.default_rng(seed).standard_normal((n1, n2)).astype(dt)
    want = F.fkdip(d, w)
    got = emu(d, w)
    assert rel_l2(got, want) <= (TOL64 if dt == np.float64 else TOL32)
