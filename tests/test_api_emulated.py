"""The host layer of the coherence, painting and sparse-interpolation rows
(argument handling, flattening, reshapes, the parabolic hmax state) through
the GPU tests' own checks, on the CPU: the three device wrappers are replaced, for these tests
only, by the kernels' per-thread code run on the CPU (tests/emu), and the
host-to-device copy by a CPU tensor.  The library itself has no CPU path."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

torch = pytest.importorskip("torch")

HERE = os.path.dirname(os.path.abspath(__file__))
P, I, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_float


def _build(tmp, name):
    so = str(tmp / f"lib{name}.so")
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-std=c++17", "-o", so,
                    os.path.join(HERE, "emu", f"{name}.cpp")], check=True)
    return ctypes.CDLL(so)


@pytest.fixture(scope="module")
def emulated(tmp_path_factory):
    tmp = tmp_path_factory.mktemp("api_emu")
    coh, paint, sint = _build(tmp, "coh_emu"), _build(tmp, "paint_emu"), _build(tmp, "sint_emu")
    coh.emu_coherence.argtypes = [P, P, P, I, I, I, I, F, I, F, P]
    coh.emu_coherence_batch.argtypes = [P, P, P, I, I, I, I, I, F, I, F, P]
    paint.emu_paint2d.argtypes = [P, P, P, I, I, I, I, F]
    paint.emu_paint2d_batch.argtypes = [P, P, P, I, I, I, I, I, F]
    sint.emu_sint2d.argtypes = [P, P, P, P, I, I, I, I, I, F]
    return coh, paint, sint


@pytest.fixture
def ps(emulated, monkeypatch):
    from pyseistr_gb300 import api
    from pyseistr_gb300 import device as D

    coh, paint, sint = emulated
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731

    def to_flat(a):
        if isinstance(a, torch.Tensor):
            t = a.to(dtype=torch.float32)
            return t.permute(*reversed(range(t.dim()))).contiguous().view(-1), True
        arr = np.asarray(a, dtype=np.float32)
        return torch.from_numpy(np.ascontiguousarray(arr.reshape(-1, order="F"))), False

    def coherence(x, v, h, typ, nt, dt, forw, hmax, out=None):
        nv, nh = v.numel(), h.numel()
        assert x.numel() == nt * (nv if forw == 1 else nh) and x.is_contiguous()
        out = torch.empty(nt * (nh if forw == 1 else nv), dtype=torch.float32)
        assert coh.emu_coherence(ptr(x), ptr(v), ptr(h), int(typ), int(nt), nv, nh, float(dt),
                                 int(forw), float(hmax), ptr(out)) == 0
        return out

    def paint2d(dip, seed, n1, n2, order, i0, eps, out=None, workspace=None):
        assert dip.numel() == n1 * n2 and seed.numel() == n1 and seed.is_contiguous()
        out = torch.empty(n1 * n2, dtype=torch.float32)
        assert paint.emu_paint2d(ptr(dip), ptr(seed), ptr(out), n1, n2, order, i0,
                                 float(eps)) == 0
        return out

    def sint2d(din, dip, mask, n1, n2, niter, ns, order, eps, out=None, workspace=None):
        n = n1 * n2
        assert din.numel() == n and dip.numel() == n and mask.numel() == n
        assert dip.is_contiguous() and mask.is_contiguous()
        out = torch.empty(n, dtype=torch.float32)
        assert sint.emu_sint2d(ptr(din), ptr(dip), ptr(mask), ptr(out), n1, n2, niter, ns,
                               order, float(eps)) == 0
        return out

    monkeypatch.setattr(api, "_to_dev_flat", to_flat)
    monkeypatch.setattr(D, "sint2d", sint2d)
    def coherence_batch(x, v, h, typ, nt, nwin, dt, forw, hmax, out=None):
        nv, nh = v.numel(), h.numel()
        assert x.numel() == nwin * nt * (nv if forw == 1 else nh) and x.is_contiguous()
        out = torch.empty(nwin * nt * (nh if forw == 1 else nv), dtype=torch.float32)
        assert coh.emu_coherence_batch(ptr(x), ptr(v), ptr(h), int(typ), int(nt), nv, nh,
                                       int(nwin), float(dt), int(forw), float(hmax),
                                       ptr(out)) == 0
        return out

    monkeypatch.setattr(D, "coherence", coherence)
    monkeypatch.setattr(D, "coherence_batch", coherence_batch)
    def paint2d_batch(dip, seed, n1, n2, nsec, order, i0, eps, out=None, workspace=None):
        assert dip.numel() == nsec * n1 * n2 and seed.numel() == nsec * n1
        assert dip.is_contiguous() and seed.is_contiguous()
        out = torch.empty(nsec * n1 * n2, dtype=torch.float32)
        assert paint.emu_paint2d_batch(ptr(dip), ptr(seed), ptr(out), n1, n2, nsec, order, i0,
                                       float(eps)) == 0
        return out

    monkeypatch.setattr(D, "paint2d", paint2d)
    monkeypatch.setattr(D, "paint2d_batch", paint2d_batch)
    import pyseistr_gb300

    return pyseistr_gb300


def test_coherence_api(ps):
    import test_gpu_zcoherence as T

    T.test_cohc_fb_matches_reference_in_call_order(ps)
    for c in T.CASES[1:]:  # the first, a DAS window's shape, is left to the GPU run
        T.test_cohc_matches_oracle(ps, c)
    T.test_cohc_refuses_what_the_reference_cannot_compute(ps)
    T.test_cohc_batch_equals_one_call_per_window(ps)


def test_painting_api(ps):
    import test_gpu_zpaint as T

    T.test_pwpaintc_matches_reference(ps)
    for c in T.CASES:
        T.test_rgt_matches_oracle(ps, c)
    T.test_cpaint2d_refuses_bad_arguments(ps)
    T.test_pwpaintc_batch_equals_one_call_per_section(ps)
    rng = np.random.default_rng(21)
    dip = rng.standard_normal((80, 30)).astype(np.float32)
    tr = rng.standard_normal(80).astype(np.float32)
    a = ps.pwpaintc(dip, tr, order=2, i0=10, eps=0.1)
    b = ps.pwpaintc(torch.from_numpy(dip), torch.from_numpy(tr), order=2, i0=10, eps=0.1)
    assert tuple(b.shape) == (80, 30) and np.array_equal(b.numpy(), a)


def test_sparse_interpolation_api(ps):
    import test_gpu_zsint as T

    T.test_sint2dc_matches_reference(ps)
    for c in T.CASES[1:]:  # the first, a 501 x 100 section, is left to the GPU run
        T.test_sint2dc_matches_oracle(ps, c)
    T.test_csint2d_refuses_bad_arguments(ps)
    d, mask, dip = T._case(80, 24, 0.4, 21)
    a = ps.sint2dc(d, mask, dip, niter=12, ns=2, order=2)
    b = ps.sint2dc(torch.from_numpy(d), torch.from_numpy(mask), torch.from_numpy(dip),
                   niter=12, ns=2, order=2)
    assert tuple(b.shape) == (80, 24) and np.array_equal(b.numpy(), a)


def test_sparse_interpolation_3d_api(ps, emulated, monkeypatch):
    from pyseistr_gb300 import device as D

    sint = emulated[2]
    sint.emu_sint3d.argtypes = [P] * 5 + [I] * 8 + [F]
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731

    def sint3d(din, dipi, dipx, mask, n, niter, ns, order, eps, out=None, workspace=None):
        m = n[0] * n[1] * n[2]
        assert all(t.numel() == m and t.is_contiguous() for t in (din, dipi, dipx, mask))
        out = torch.empty(m, dtype=torch.float32)
        assert sint.emu_sint3d(ptr(din), ptr(dipi), ptr(dipx), ptr(mask), ptr(out), *n, niter,
                               *ns, *order, float(eps)) == 0
        return out

    monkeypatch.setattr(D, "sint3d", sint3d)
    import test_gpu_zsint as T

    T.test_sint3dc_matches_reference(ps)
    for c in T.CASES3[1:]:
        T.test_sint3dc_matches_oracle(ps, c)


def test_fk_api(ps, tmp_path, monkeypatch):
    from pyseistr_gb300 import device as D

    lib = _build(tmp_path, "fk_emu")
    D_ = ctypes.c_double
    lib.emu_fkdip.argtypes = lib.emu_fkdip_f64.argtypes = [P, P, I, I, D_]
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731

    def fkdip(d, n1, n2, w, out=None, workspace=None):
        assert d.numel() == n1 * n2 and d.is_contiguous()
        assert d.dtype in (torch.float32, torch.float64)
        out = torch.empty(n1 * n2, dtype=torch.float64)
        fn = lib.emu_fkdip_f64 if d.dtype == torch.float64 else lib.emu_fkdip
        assert fn(ptr(d), ptr(out), n1, n2, float(w)) == 0
        return out

    monkeypatch.setattr(D, "fkdip", fkdip)
    monkeypatch.setattr(api_module(), "_dev", lambda: torch.device("cpu"))
    import test_gpu_zfk as T

    T.test_fkdip_matches_reference(ps)
    for c in T.CASES[1:]:
        T.test_fkdip_matches_oracle(ps, c)
    T.test_fkdip_zero_width_raises_like_the_reference(ps)
    d = np.random.default_rng(21).standard_normal((200, 64)).astype(np.float32)
    a = ps.fkdip(d, 0.05)
    b = ps.fkdip(torch.from_numpy(d), 0.05)
    assert b.dtype == torch.float64 and np.array_equal(b.numpy(), a)
    e = np.random.default_rng(22).standard_normal((200, 64)).astype(np.float32)
    both = ps.fkdip((2 * d - 3 * e).astype(np.float32), 0.05)
    assert T.rel_l2(both, 2 * a - 3 * ps.fkdip(e, 0.05)) <= 1e-5


def api_module():
    from pyseistr_gb300 import api

    return api
