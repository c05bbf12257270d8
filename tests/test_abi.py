"""The C-ABI library loads and exports every entry point include/pwd_gb300.h
declares; host-side argument checks and workspace queries (no GPU needed)."""
import ctypes
import os
import re

import pytest

from pyseistr_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "pwd_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pwd_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ("pwd_dip", "pwd_somean2d", "pwd_somf2d", "pwd_somean3d", "pwd_somf3d",
              "pwd_soint3d"):
        assert n in names and n + "_workspace_size" in names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_status_strings_and_version():
    lib = _lib.load()
    assert lib.pwd_version() >= 100
    for s in range(5):
        assert lib.pwd_status_string(s)
    with pytest.raises(ValueError):
        _lib.check(_lib.PWD_EINVAL, "x")
    with pytest.raises(_lib.PwdError):
        _lib.check(_lib.PWD_EWORKSPACE, "x")


def test_workspace_queries():
    lib = _lib.load()
    rect = (ctypes.c_int * 3)(10, 10, 1)
    a = lib.pwd_dip_workspace_size(501, 100, 1, 2, rect, 0)
    b = lib.pwd_dip_workspace_size(501, 100, 1, 2, rect, 1)
    assert a >= 11 * 501 * 100 * 4 and b > a
    assert lib.pwd_dip_workspace_size(0, 100, 1, 2, rect, 0) == 0
    assert lib.pwd_somean2d_workspace_size(501, 100, 1, 8, 2) >= 17 * 501 * 100 * 4
    assert lib.pwd_somf2d_workspace_size(501, 100, 1, 8, 17, 1, 2) > 0
    assert lib.pwd_somf2d_workspace_size(501, 100, 1, 8, 0, 1, 2) == 0   # empty window
    assert lib.pwd_somf2d_workspace_size(501, 100, 1, 1, 3, 2, 2) == 0   # svmf needs nmf >= 5
    assert lib.pwd_somean3d_workspace_size(201, 60, 60, 4, 4, 2) >= 81 * 201 * 3600 * 4
    assert lib.pwd_somean3d_workspace_size(201, 60, 60, 11, 4, 2) == 0   # radius cap
    assert lib.pwd_soint3d_workspace_size(64, 32, 32, 2) > 0
    assert lib.pwd_soint3d_workspace_size(64, 32, 32, 9) == 0


def test_calls_reject_bad_arguments_before_touching_the_gpu():
    lib = _lib.load()
    rect = (ctypes.c_int * 3)(10, 10, 1)
    fake = ctypes.c_void_p(256)  # never dereferenced: rejected by the host checks
    assert lib.pwd_dip(None, None, fake, 10, 10, 1, 5, 10, 2, rect, fake, 1 << 20, None) == _lib.PWD_EINVAL
    assert lib.pwd_dip(fake, None, fake, 10, 10, 1, 5, 10, 9, rect, fake, 1 << 20, None) == _lib.PWD_ENOTSUP
    assert lib.pwd_dip(fake, None, fake, 4, 10, 1, 5, 10, 2, rect, fake, 1 << 20, None) == _lib.PWD_EINVAL
    assert lib.pwd_dip(fake, None, fake, 100, 10, 1, 5, 10, 2, rect, fake, 16, None) == _lib.PWD_EWORKSPACE
    assert lib.pwd_dip(fake, None, fake, 100, 10, 1, 5, 10, 2, rect, ctypes.c_void_p(300), 1 << 30, None) == _lib.PWD_EWORKSPACE
    assert lib.pwd_somean2d(fake, fake, fake, 3, 10, 1, 2, 2, 0, 0.01, fake, 1 << 20, None) == _lib.PWD_EINVAL
    assert lib.pwd_somf2d(fake, fake, fake, 50, 10, 1, 2, 5, 1, 2, 0.01, fake, 16, None) == _lib.PWD_EWORKSPACE
    assert lib.pwd_somf3d(fake, fake, fake, fake, 50, 10, 10, 2, 2, 70000, 1, 2, 0.01, fake, 1 << 30, None) == _lib.PWD_ENOTSUP
    assert lib.pwd_soint3d(fake, None, fake, fake, fake, 8, 8, 8, 2, 1, 1, 5, 0, 1, 1, 0.0, fake, 1 << 30, None) == _lib.PWD_EINVAL


def test_patch_and_bandpass_entries_check_arguments_on_the_host():
    """pwd_patch_count is host arithmetic; invalid sizes and null pointers
    come back as PWD_EINVAL before any launch."""
    from oracle import patch_oracle as P

    lib = _lib.load()
    fake = ctypes.c_void_p(256)
    for n, l, s in [((37, 29, 1), (8, 8, 1), (4, 4, 1)), ((13, 11, 9), (4, 4, 4), (2, 2, 2)),
                    ((5, 30, 1), (8, 6, 1), (4, 3, 1)), ((2000, 5000, 1), (64, 64, 1), (32, 32, 1))]:
        want = 1
        for a in range(3):
            want *= len(P.starts(n[a], l[a], s[a]))
        assert lib.pwd_patch_count(*n, *l, *s) == want
    assert lib.pwd_patch_count(8, 8, 1, 0, 4, 1, 2, 2, 1) == 0  # zero window
    assert lib.pwd_patch_count(3, 40, 7, 5, 8, 2, 2, 6, 3) == 0  # an axis with no window
    assert lib.pwd_patch(None, fake, 8, 8, 1, 4, 4, 1, 2, 2, 1, None) == _lib.PWD_EINVAL
    assert lib.pwd_patch(fake, fake, 8, 8, 1, 4, 4, 1, 0, 2, 1, None) == _lib.PWD_EINVAL
    assert lib.pwd_patch_inv(fake, None, 8, 8, 1, 4, 4, 1, 2, 2, 1, None) == _lib.PWD_EINVAL
    assert lib.pwd_bandpass(None, fake, 100, 3, 1, 0.004, 0.0, 20.0, 6, 6, 0, None) == _lib.PWD_EINVAL
    assert lib.pwd_bandpass(fake, fake, 0, 3, 1, 0.004, 0.0, 20.0, 6, 6, 0, None) == _lib.PWD_EINVAL
    assert lib.pwd_bandpass(fake, fake, 100, 3, 0, 0.004, 0.0, 20.0, 6, 6, 0, None) == _lib.PWD_EINVAL
    # in place with no cut at all: nothing to do, no CUDA call
    assert lib.pwd_bandpass(fake, fake, 100, 3, 1, 0.004, 0.0, 125.0, 6, 6, 0, None) == _lib.PWD_OK


def test_coherence_entry_checks_arguments_on_the_host():
    """Null pointers, empty sizes and an operator other than 1 / -1 come back
    as PWD_EINVAL before any launch."""
    lib = _lib.load()
    fake = ctypes.c_void_p(256)
    ok = _lib.PWD_EINVAL
    assert lib.pwd_coherence(None, fake, fake, 1, 10, 2, 2, 0.004, -1, 0.0, fake, None) == ok
    assert lib.pwd_coherence(fake, fake, fake, 1, 0, 2, 2, 0.004, -1, 0.0, fake, None) == ok
    assert lib.pwd_coherence(fake, fake, fake, 1, 10, 0, 2, 0.004, 1, 0.0, fake, None) == ok
    assert lib.pwd_coherence(fake, fake, fake, 1, 10, 2, 0, 0.004, 1, 0.0, fake, None) == ok
    assert lib.pwd_coherence(fake, fake, fake, 2, 10, 2, 2, 0.004, 0, 0.0, fake, None) == ok
    assert lib.pwd_coherence_batch(fake, fake, fake, 1, 10, 2, 2, 0, 0.004, -1, 0.0, fake, None) == ok


def test_paint_entry_checks_arguments_on_the_host():
    """Workspace query and argument checks of pwd_paint2d, before any launch."""
    lib = _lib.load()
    fake = ctypes.c_void_p(256)
    assert lib.pwd_paint2d_workspace_size(3, 2) == 0
    assert lib.pwd_paint2d_workspace_size(100, 5) == 0
    need = lib.pwd_paint2d_workspace_size(100, 2)
    assert need >= 2 * 15 * 100 * 4 and need % 256 == 0
    assert lib.pwd_paint2d(fake, fake, fake, 100, 10, 2, 10, 0.1, fake, need, None) == _lib.PWD_EINVAL
    assert lib.pwd_paint2d(fake, fake, fake, 100, 10, 2, -1, 0.1, fake, need, None) == _lib.PWD_EINVAL
    assert lib.pwd_paint2d(fake, fake, fake, 3, 10, 2, 0, 0.1, fake, need, None) == _lib.PWD_EINVAL
    assert lib.pwd_paint2d(fake, fake, fake, 100, 10, 5, 0, 0.1, fake, need, None) == _lib.PWD_ENOTSUP
    assert lib.pwd_paint2d(fake, fake, fake, 100, 10, 2, 0, 0.1, fake, need - 256, None) == _lib.PWD_EWORKSPACE
    assert lib.pwd_paint2d(fake, fake, fake, 100, 10, 2, 0, 0.1, ctypes.c_void_p(300), need, None) == _lib.PWD_EWORKSPACE
    assert lib.pwd_paint2d_batch_workspace_size(100, 3, 2) >= 3 * (need - 256)
    assert lib.pwd_paint2d_batch(fake, fake, fake, 100, 10, 0, 2, 0, 0.1, fake, need, None) == _lib.PWD_EINVAL
    assert lib.pwd_paint2d_batch(fake, fake, fake, 100, 10, 3, 2, 0, 0.1, fake, need, None) == _lib.PWD_EWORKSPACE


def test_sint_entry_checks_arguments_on_the_host():
    lib = _lib.load()
    fake = ctypes.c_void_p(256)
    assert lib.pwd_sint2d_workspace_size(3, 10, 1, 1) == 0
    assert lib.pwd_sint2d_workspace_size(40, 10, 1, 5) == 0
    need = lib.pwd_sint2d_workspace_size(40, 10, 2, 2)
    assert need >= 8 * 40 * 10 * 4 + lib.pwd_somean2d_workspace_size(40, 10, 1, 2, 2)
    assert lib.pwd_sint2d(None, fake, fake, fake, 40, 10, 5, 1, 1, 0.01, fake, need, None) == _lib.PWD_EINVAL
    assert lib.pwd_sint2d(fake, fake, fake, fake, 40, 10, -1, 1, 1, 0.01, fake, need, None) == _lib.PWD_EINVAL
    assert lib.pwd_sint2d(fake, fake, fake, fake, 40, 10, 5, 1, 5, 0.01, fake, need, None) == _lib.PWD_ENOTSUP
    assert lib.pwd_sint2d(fake, fake, fake, fake, 40, 10, 5, 2, 2, 0.01, fake, need - 256, None) == _lib.PWD_EWORKSPACE
    need3 = lib.pwd_sint3d_workspace_size(24, 5, 6, 1, 2, 2, 1)
    assert need3 >= 12 * 24 * 5 * 6 * 4
    assert lib.pwd_sint3d_workspace_size(24, 5, 6, 1, 2, 2, 5) == 0
    assert lib.pwd_sint3d(fake, fake, fake, fake, fake, 24, 5, 0, 5, 1, 1, 1, 1, 0.01, fake, need3, None) == _lib.PWD_EINVAL
    assert lib.pwd_sint3d(fake, fake, fake, fake, fake, 24, 5, 6, 5, 1, 2, 2, 1, 0.01, fake, need3 - 256, None) == _lib.PWD_EWORKSPACE


def test_fk_entry_checks_arguments_on_the_host():
    lib = _lib.load()
    fake = ctypes.c_void_p(256)
    need = lib.pwd_fkdip_workspace_size(100, 30, 0)
    need64 = lib.pwd_fkdip_workspace_size(100, 30, 1)
    assert need > 0 and need64 > need and need % 256 == 0
    assert lib.pwd_fkdip_workspace_size(0, 30, 0) == 0
    assert lib.pwd_fkdip(fake, fake, 100, 30, 0.0, fake, need, None) == _lib.PWD_EINVAL
    assert lib.pwd_fkdip(None, fake, 100, 30, 0.05, fake, need, None) == _lib.PWD_EINVAL
    assert lib.pwd_fkdip(fake, fake, 100, 30, 0.05, fake, need - 256, None) == _lib.PWD_EWORKSPACE
    assert lib.pwd_fkdip_f64(fake, fake, 100, 30, 0.05, fake, need, None) == _lib.PWD_EWORKSPACE
