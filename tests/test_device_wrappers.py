"""The device-level wrappers of the coherence, painting, sparse-interpolation
and FK entries (pyseistr_gb300/device.py) on the CPU, against a stand-in for
the library that checks every call's arguments against the ctypes signature
of the C entry (count and convertibility) and runs no kernel.  This covers
the wrappers' own host code: sizes, workspace queries, argument order."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")


class FakeLib:
    def __init__(self, sigs):
        self.sigs = sigs
        self.calls = []

    def __getattr__(self, name):
        argtypes, restype = self.sigs[name]

        def call(*args):
            assert len(args) == len(argtypes), (name, len(args), len(argtypes))
            for a, t in zip(args, argtypes):
                if t is ctypes.c_void_p:
                    assert a is None or isinstance(a, ctypes.c_void_p), (name, a)
                else:
                    t(a)  # raises if the value does not convert
            self.calls.append((name, args))
            return 1 << 20 if name.endswith("_workspace_size") else 0

        return call


@pytest.fixture
def fake(monkeypatch):
    from pyseistr_gb300 import _lib
    from pyseistr_gb300 import device as D

    lib = FakeLib(_lib.SIGNATURES)
    monkeypatch.setattr(_lib, "load", lambda *a, **k: lib)

    def as_flat(t, n, name):
        assert isinstance(t, torch.Tensor) and t.numel() == n, (name, t.numel(), n)
        return t

    monkeypatch.setattr(D, "_as_flat", as_flat)
    monkeypatch.setattr(D, "_stream", lambda: None)
    return lib, D


def _f(n, dtype=torch.float32):
    return torch.zeros(n, dtype=dtype)


def test_coherence_wrapper(fake):
    lib, D = fake
    out = D.coherence(_f(50 * 8), _f(5), _f(8), 1, 50, 0.004, -1, 0.0)
    assert out.numel() == 50 * 5
    out = D.coherence(_f(50 * 5), _f(5), _f(8), 2, 50, 0.004, 1, 3.0)
    assert out.numel() == 50 * 8
    assert [c[0] for c in lib.calls] == ["pwd_coherence"] * 2
    out = D.coherence_batch(_f(3 * 50 * 8), _f(5), _f(8), 1, 50, 3, 0.004, -1, 0.0)
    assert out.numel() == 3 * 50 * 5 and lib.calls[-1][0] == "pwd_coherence_batch"


def test_paint_wrapper(fake):
    lib, D = fake
    out = D.paint2d(_f(40 * 9), _f(40), 40, 9, 2, 3, 0.1)
    assert out.numel() == 40 * 9
    assert [c[0] for c in lib.calls] == ["pwd_paint2d_workspace_size", "pwd_paint2d"]
    out = D.paint2d_batch(_f(3 * 40 * 9), _f(3 * 40), 40, 9, 3, 2, 3, 0.1)
    assert out.numel() == 3 * 40 * 9 and lib.calls[-1][0] == "pwd_paint2d_batch"


def test_sint_wrappers(fake):
    lib, D = fake
    assert D.sint2d(_f(40 * 9), _f(40 * 9), _f(40 * 9), 40, 9, 5, 1, 2, 0.01).numel() == 360
    n = 16 * 5 * 4
    assert D.sint3d(_f(n), _f(n), _f(n), _f(n), (16, 5, 4), 5, (1, 2), (2, 1), 0.01).numel() == n
    assert [c[0] for c in lib.calls] == ["pwd_sint2d_workspace_size", "pwd_sint2d",
                                         "pwd_sint3d_workspace_size", "pwd_sint3d"]


def test_fk_wrapper(fake, monkeypatch):
    lib, D = fake
    cuda_like = _f(30 * 7)
    monkeypatch.setattr(torch.Tensor, "is_cuda", property(lambda self: True))
    out = D.fkdip(cuda_like, 30, 7, 0.05)
    assert out.dtype == torch.float64 and out.numel() == 210
    D.fkdip(_f(30 * 7, torch.float64), 30, 7, 0.05)
    names = [c[0] for c in lib.calls]
    assert names == ["pwd_fkdip_workspace_size", "pwd_fkdip", "pwd_fkdip_workspace_size",
                     "pwd_fkdip_f64"]
    assert lib.calls[2][1][2] == 1  # the double entry's workspace
