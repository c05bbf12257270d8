"""pwd_dip_static: slope estimation for callers that cannot allocate device
memory (a plugin inside an application that owns the CUDA context and its
memory budget, a real-time loop that must not call cudaMalloc after
start-up).  It keeps its scratch in a fixed device array inside the library
instead of a caller workspace.  This test calls it through the C ABI, twice
in a row, and requires the results of the workspace entry point pwd_dip.

The file sorts last so that a run stopping at the first failure has run
every other test before it; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from gpu_util import DIP_TOL, need_gpu, rel_l2

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def test_dip_static_equals_dip_on_two_calls():
    need_gpu()
    import torch

    import workloads
    from pyseistr_gb300 import _lib
    from pyseistr_gb300 import device as D

    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    d = workloads.plain2d()  # 501 x 100
    n1, n2 = d.shape
    data = torch.from_numpy(np.ascontiguousarray(d.reshape(-1, order="F"))).cuda()
    want = D.dip(data, n1, n2, 1, 5, 10, 2, (10, 10, 1)).cpu().numpy()

    cube = workloads.plain3d()[:64, :20, :16].copy()
    c = torch.from_numpy(np.ascontiguousarray(cube.reshape(-1, order="F"))).cuda()
    want3 = D.dip(c, 64, 20, 16, 3, 6, 2, (5, 5, 5)).cpu().numpy()

    rect = (ctypes.c_int * 3)(10, 10, 1)
    rect3 = (ctypes.c_int * 3)(5, 5, 5)
    for _ in range(2):  # the array keeps the previous call's contents
        out = torch.full((n1 * n2,), float("nan"), device="cuda")
        rc = lib.pwd_dip_static(_ptr(data), None, _ptr(out), n1, n2, 1, 5, 10, 2, rect, stream)
        assert rc == _lib.PWD_OK
        out3 = torch.full((2 * cube.size,), float("nan"), device="cuda")
        rc = lib.pwd_dip_static(_ptr(c), None, _ptr(out3), 64, 20, 16, 3, 6, 2, rect3, stream)
        assert rc == _lib.PWD_OK
        torch.cuda.synchronize()
        got, got3 = out.cpu().numpy(), out3.cpu().numpy()
        assert np.isfinite(got).all() and np.isfinite(got3).all()
        assert rel_l2(got, want) <= DIP_TOL and rel_l2(got3, want3) <= DIP_TOL
        assert np.array_equal(got, want) and np.array_equal(got3, want3)


def test_dip_static_rejects_sections_beyond_its_capacity():
    need_gpu()
    from pyseistr_gb300 import _lib

    lib = _lib.load()
    cap = lib.pwd_dip_static_capacity()
    assert cap == 64 << 20
    rect = (ctypes.c_int * 3)(10, 10, 1)
    fake = ctypes.c_void_p(256)  # never touched: the size check comes first
    # 2000 x 2000 needs about 200 MB of scratch
    assert lib.pwd_dip_workspace_size(2000, 2000, 1, 2, rect, 0) > cap
    rc = lib.pwd_dip_static(fake, None, fake, 2000, 2000, 1, 5, 10, 2, rect, None)
    assert rc == _lib.PWD_EWORKSPACE
