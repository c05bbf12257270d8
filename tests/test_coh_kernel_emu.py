"""The coherence kernels' per-thread code (pwd_coh.cuh) run on the CPU for
every thread of their grids (tests/emu/coh_emu.cpp) against the oracle and
the reference's own outputs (golden_coh.npz): bit for bit, and, where the
oracle leaves a sample undefined (the reference reads past the end of its
data), the value with that sample read as 0.  The GPU runs the same code in
tests/test_gpu_zcoherence.py."""
import ctypes
import json
import os
import subprocess

import numpy as np
import pytest

from coh_util import agrees
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "golden_coh.npz")


@pytest.fixture(scope="module")
def emu(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("coh_emu") / "libcoh_emu.so")
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-std=c++17", "-o", so,
                    os.path.join(HERE, "emu", "coh_emu.cpp")], check=True)
    lib = ctypes.CDLL(so)
    P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    lib.emu_coherence.argtypes = [P, P, P, I, I, I, I, F, I, F, P]
    lib.emu_coherence.restype = I

    def run(x, v, h, typ, nt, dt, forw, hmax):
        x = np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1, order="F"))
        v = np.ascontiguousarray(v, np.float32)
        h = np.ascontiguousarray(h, np.float32)
        out = np.full(nt * (h.size if forw == 1 else v.size), 7.0, np.float32)
        p = lambda a: a.ctypes.data_as(P)  # noqa: E731
        assert lib.emu_coherence(p(x), p(v), p(h), typ, nt, v.size, h.size, dt, forw,
                                 float(hmax), p(out)) == 0
        return out

    return run


def test_emulated_kernels_match_reference_and_oracle(emu):
    """The fixture's calls in order with one oracle object, whose hmax after
    each call is the one the reference used."""
    z = np.load(GOLDEN)
    op = O.Coherence()
    for m in json.loads(bytes(z["meta"]).decode()):
        k = m["k"]
        x, v, h = z[f"in_{k}"], z[f"v_{k}"], z[f"h_{k}"]
        want = op(x, v, h, m["typ"], m["nt"], m["dt"], m["forw"]).reshape(-1, order="F")
        got = emu(x, v, h, m["typ"], m["nt"], m["dt"], m["forw"], op.hmax[0])
        assert agrees(got, want, x, v, h, m["typ"], m["nt"], m["dt"], op.hmax[0]), k
        ref = z[f"out_{k}"]
        ok = ~np.isnan(want)
        assert np.array_equal(got[ok], ref[ok]), k
        assert np.isfinite(got).all(), k


def _carry_terms(v, h, nt, dt):
    """Linear curves of traces other than the last that reach sample nt (the
    next trace's first sample), in float32 as the kernels compute them."""
    f32 = np.float32
    itau = np.arange(nt, dtype=f32)[:, None, None]
    t = itau * f32(dt) + h[None, :-1, None] * v[None, None, :]
    it = np.floor(t / f32(dt)) + f32(1)
    return int((it == nt).sum())


CASES = [
    # typ, nt, nv, nh, dt, forw, seed, v range, h range
    (1, 300, 100, 96, 0.0005, -1, 1, (-0.005, 0.005), (0.0, 95.0)),
    (1, 300, 100, 96, 0.0005, 1, 2, (-0.005, 0.005), (0.0, 95.0)),
    (1, 97, 13, 21, 0.004, 1, 3, (-0.02, 0.03), (-40.0, 60.0)),
    (1, 97, 13, 21, 0.004, -1, 4, (-0.02, 0.03), (-40.0, 60.0)),
    (2, 64, 9, 17, 0.004, 1, 5, (-0.1, 0.2), (-30.0, 50.0)),
    (2, 64, 9, 17, 0.004, -1, 6, (-0.1, 0.2), (-30.0, 50.0)),
    (3, 120, 11, 15, 0.002, 1, 7, (1500.0, 4000.0), (-300.0, 400.0)),
    (3, 120, 11, 15, 0.002, -1, 8, (1500.0, 4000.0), (-300.0, 400.0)),
    (7, 50, 5, 6, 0.004, -1, 9, (-0.01, 0.01), (0.0, 5.0)),  # unknown type: linear
    (2, 80, 6, 9, 0.004, -1, 12, (-0.2, 0.1), (-60.0, 20.0)),  # negative hmax state
    (3, 60, 7, 9, 0.002, 1, 13, (-3000.0, -1500.0), (-100.0, 100.0)),  # negative velocities
    (1, 1, 1, 1, 0.004, 1, 10, (0.0, 0.0), (0.0, 0.0)),
    (1, 1, 1, 1, 0.004, -1, 11, (0.0, 0.0), (0.0, 0.0)),
]


@pytest.mark.parametrize("case", CASES, ids=[f"typ{c[0]}-{c[1]}x{c[2]}x{c[3]}-f{c[5]}"
                                             for c in CASES])
def test_emulated_kernels_match_oracle(emu, case):
    typ, nt, nv, nh, dt, forw, seed, vr, hr = case
    rng = np.random.default_rng(seed)
    v = np.sort(rng.uniform(*vr, nv)).astype(np.float32)
    h = np.sort(rng.uniform(*hr, nh)).astype(np.float32)
    x = rng.standard_normal((nt, nv if forw == 1 else nh)).astype(np.float32)
    op = O.Coherence()
    want = op(x, v, h, typ, nt, dt, forw).reshape(-1, order="F")
    got = emu(x, v, h, typ, nt, dt, forw, op.hmax[0])
    assert agrees(got, want, x, v, h, typ, nt, dt, op.hmax[0])
    assert np.isfinite(got).all()


def test_forward_cases_reach_the_next_trace():
    """The linear forward cases above do exercise the terms that land on the
    next trace's first sample."""
    for typ, nt, nv, nh, dt, forw, seed, vr, hr in CASES:
        if typ == 1 and forw == 1 and nh > 1:
            rng = np.random.default_rng(seed)
            v = np.sort(rng.uniform(*vr, nv)).astype(np.float32)
            h = np.sort(rng.uniform(*hr, nh)).astype(np.float32)
            assert _carry_terms(v, h, nt, dt) > 0


REFUSALS = [
    # typ, v, h, nt, dt: cases the oracle refuses (no usable sample index) and not
    (3, [0.0, 1000.0], [0.0, 10.0], 20, 0.004),     # h / v = 0 / 0
    (3, [0.0, 1000.0], [5.0, 10.0], 20, 0.004),     # h / v = inf
    (1, [0.01], [1.0], 20, 0.0),                    # t / 0
    (1, [3.0e5], [3.0e5], 20, 0.004),               # beyond 2e9 samples
    (1, [-0.01, 0.01], [0.0, 1.0], 20, 0.004),      # usable
    (3, [1500.0, 3000.0], [-100.0, 100.0], 20, 0.004),
    (2, [0.1, 0.2], [0.0, 0.0], 20, 0.004),          # hmax 0: 0 / 0
]


@pytest.mark.parametrize("case", REFUSALS)
def test_host_index_check_agrees_with_oracle(case):
    """The host check before a launch refuses exactly the calls the oracle
    refuses, with the hmax the call uses."""
    from pyseistr_gb300 import api

    typ, v, h, nt, dt = case
    v, h = np.asarray(v, np.float32), np.asarray(h, np.float32)
    op = O.Coherence()
    x = np.ones((nt, h.size), np.float32)
    try:
        op(x, v, h, typ, nt, dt, -1)
        refused = False
    except ValueError:
        refused = True
    st = api._CohState()
    if typ == 2:
        st.update(h)
    assert api._coh_indices_usable(v, h, typ, nt, dt, st.hmax) == (not refused)


def test_hmax_state_follows_the_reference_static():
    """hmax carried across parabolic calls as coh_init2 updates its static:
    set to the signed offset h[i] whenever hmax < |h[i]|, never reset."""
    from pyseistr_gb300 import api

    rng = np.random.default_rng(12)
    op = O.Coherence()
    st = api._CohState()
    for _ in range(6):
        h = rng.uniform(-50, 50, int(rng.integers(1, 9))).astype(np.float32)
        v = np.array([0.1, 0.2], np.float32)
        op(np.zeros((8, h.size), np.float32), v, h, 2, 8, 0.004, -1)
        st.update(h)
        assert st.hmax == op.hmax[0]


@pytest.mark.parametrize("forw", [-1, 1])
def test_emulated_stacked_windows_equal_one_call_per_window(tmp_path, forw):
    """The batch decomposition (window of each thread) over 3 stacked
    windows gives each window's single-call result."""
    so = str(tmp_path / "libcoh_emu.so")
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-std=c++17", "-o", so,
                    os.path.join(HERE, "emu", "coh_emu.cpp")], check=True)
    lib = ctypes.CDLL(so)
    P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    lib.emu_coherence_batch.argtypes = [P, P, P, I, I, I, I, I, F, I, F, P]
    rng = np.random.default_rng(40)
    nt, nv, nh, nwin = 90, 11, 17, 3
    v = np.sort(rng.uniform(-0.01, 0.01, nv)).astype(np.float32)
    h = np.arange(nh, dtype=np.float32)
    wins = [rng.standard_normal((nt, nv if forw == 1 else nh)).astype(np.float32)
            for _ in range(nwin)]
    x = np.ascontiguousarray(np.concatenate([w.reshape(-1, order="F") for w in wins]))
    out = np.full(nwin * nt * (nh if forw == 1 else nv), 7.0, np.float32)
    p = lambda a: a.ctypes.data_as(P)  # noqa: E731
    assert lib.emu_coherence_batch(p(x), p(v), p(h), 1, nt, nv, nh, nwin, 0.004, forw, 0.0,
                                   p(out)) == 0
    m = out.size // nwin
    for k, w in enumerate(wins):
        want = O.Coherence()(w, v, h, 1, nt, 0.004, forw).reshape(-1, order="F")
        assert agrees(out[k * m:(k + 1) * m], want, w, v, h, 1, nt, 0.004, 0.0), k
