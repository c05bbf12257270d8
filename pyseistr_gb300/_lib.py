"""ctypes binding of libpwd_gb300.so (the C ABI declared in include/pwd_gb300.h).

The library is the only compute path: if it cannot be loaded, every entry
point raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpwd_gb300.so")

PWD_OK, PWD_EINVAL, PWD_EWORKSPACE, PWD_ECUDA, PWD_ENOTSUP = range(5)
FAMILIES = ["pwd", "cg", "triangle", "spray", "filter", "soint", "other"]

# Every symbol the header declares, with its ctypes signature.
_P, _I, _F, _S = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_size_t
SIGNATURES = {
    "pwd_version": ([], _I),
    "pwd_status_string": ([_I], ctypes.c_char_p),
    "pwd_dip_workspace_size": ([_I, _I, _I, _I, _P, _I], _S),
    "pwd_dip": ([_P, _P, _P, _I, _I, _I, _I, _I, _I, _P, _P, _S, _P], _I),
    "pwd_dip_static_capacity": ([], _S),
    "pwd_dip_static": ([_P, _P, _P, _I, _I, _I, _I, _I, _I, _P, _P], _I),
    "pwd_dip_batch_workspace_size": ([_P, _I, _I, _P, _I], _S),
    "pwd_dip_batch": ([_P, _P, _P, _P, _I, _I, _I, _I, _P, _P, _S, _P], _I),
    "pwd_dip_batch_mixed_workspace_size": ([_P, _I, _I, _P, _I], _S),
    "pwd_dip_batch_mixed": ([_P, _P, _P, _P, _I, _I, _I, _I, _P, _P, _S, _P], _I),
    "pwd_dip_batch_prepare": ([_P, _I, _I, _P, _I, _I, _P, _S, _P], _I),
    "pwd_dip_batch_run": ([_P, _P, _P, _P, _I, _I, _I, _I, _P, _I, _P, _S, _P], _I),
    "pwd_sofilter2d_batch_workspace_size": ([_P, _I, _I, _I, _I, _I, _I], _S),
    "pwd_sofilter2d_batch": ([_P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _F, _P, _S, _P], _I),
    "pwd_somean2d_workspace_size": ([_I, _I, _I, _I, _I], _S),
    "pwd_somean2d": ([_P, _P, _P, _I, _I, _I, _I, _I, _I, _F, _P, _S, _P], _I),
    "pwd_somf2d_workspace_size": ([_I, _I, _I, _I, _I, _I, _I], _S),
    "pwd_somf2d": ([_P, _P, _P, _I, _I, _I, _I, _I, _I, _I, _F, _P, _S, _P], _I),
    "pwd_somean3d_workspace_size": ([_I, _I, _I, _I, _I, _I], _S),
    "pwd_somean3d": ([_P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _F, _P, _S, _P], _I),
    "pwd_somf3d_workspace_size": ([_I, _I, _I, _I, _I, _I, _I, _I], _S),
    "pwd_somf3d": ([_P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _I, _I, _F, _P, _S, _P], _I),
    "pwd_panel_median_workspace_size": ([_I, _I, ctypes.c_long, _I, _I], _S),
    "pwd_panel_median": ([_P, _P, _I, _I, ctypes.c_long, _I, _I, _P, _S, _P], _I),
    "pwd_launch_count": ([], ctypes.c_ulonglong),
    "pwd_profile_start": ([], None),
    "pwd_profile_stop": ([_P, _P, _I], _I),
    "pwd_fp32_fma_probe": ([_P, _I, _I, _I, _P], _I),
    "pwd_patch_count": ([_I] * 9, _S),
    "pwd_patch": ([_P, _P] + [_I] * 9 + [_P], _I),
    "pwd_patch_inv": ([_P, _P] + [_I] * 9 + [_P], _I),
    "pwd_bandpass": ([_P, _P, _I, _I, _I, _F, _F, _F, _I, _I, _I, _P], _I),
    "pwd_coherence": ([_P, _P, _P, _I, _I, _I, _I, _F, _I, _F, _P, _P], _I),
    "pwd_coherence_batch": ([_P, _P, _P, _I, _I, _I, _I, _I, _F, _I, _F, _P, _P], _I),
    "pwd_paint2d_workspace_size": ([_I, _I], _S),
    "pwd_paint2d": ([_P, _P, _P, _I, _I, _I, _I, _F, _P, _S, _P], _I),
    "pwd_paint2d_batch_workspace_size": ([_I, _I, _I], _S),
    "pwd_paint2d_batch": ([_P, _P, _P, _I, _I, _I, _I, _I, _F, _P, _S, _P], _I),
    "pwd_sint2d_workspace_size": ([_I, _I, _I, _I], _S),
    "pwd_sint2d": ([_P, _P, _P, _P, _I, _I, _I, _I, _I, _F, _P, _S, _P], _I),
    "pwd_sint3d_workspace_size": ([_I] * 7, _S),
    "pwd_fkdip_workspace_size": ([_I, _I, _I], _S),
    "pwd_fkdip": ([_P, _P, _I, _I, ctypes.c_double, _P, _S, _P], _I),
    "pwd_fkdip_f64": ([_P, _P, _I, _I, ctypes.c_double, _P, _S, _P], _I),
    "pwd_sint3d": ([_P] * 5 + [_I] * 8 + [_F, _P, _S, _P], _I),
    "pwd_soint3d_workspace_size": ([_I, _I, _I, _I], _S),
    "pwd_soint3d": ([_P, _P, _P, _P, _P] + [_I] * 10 + [_F, _P, _S, _P], _I),
    "pwd_soint2d_prec_workspace_size": ([_I, _I, _I, _I], _S),
    "pwd_soint2d_prec": ([_P, _P, _P, _P, _P] + [_I] * 6 + [_P, _S, _P], _I),
    "pwd_soint2d_prec_batch_workspace_size": ([_P, _I, _I, _I], _S),
    "pwd_soint2d_prec_batch": ([_P, _P, _P, _P, _P, _P] + [_I] * 5 + [_P, _S, _P], _I),
    "pwd_soint3d_batch_workspace_size": ([_P, _I, _I], _S),
    "pwd_soint3d_batch": ([_P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I, _I, _P, _S, _P], _I),
}

_lib = None


class Section(ctypes.Structure):
    """pwd_section: one section of a batch."""
    _fields_ = [("offset", ctypes.c_long), ("out_offset", ctypes.c_long), ("n1", ctypes.c_int),
                ("n2", ctypes.c_int), ("n3", ctypes.c_int)]


class PwdError(RuntimeError):
    """A library call failed (status other than PWD_OK / PWD_EINVAL)."""


def load(build_if_missing: bool = True):
    """Load (building first if needed) and return the ctypes library."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and build_if_missing:
        from . import build as _build

        _build.build()
    if not os.path.exists(LIB_PATH):
        raise PwdError(f"CUDA extension {LIB_PATH} is missing: run pyseistr_gb300.build.build()")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(status: int, what: str) -> None:
    if status == PWD_OK:
        return
    msg = f"{what}: {load().pwd_status_string(status).decode()} (status {status})"
    if status == PWD_EINVAL:
        raise ValueError(msg)
    raise PwdError(msg)


def launch_count() -> int:
    """Kernels the library has launched since it was loaded."""
    return int(load().pwd_launch_count())


class profile:
    """Context manager timing every library launch with CUDA events:
    ``with profile() as p: ...`` then ``p.ms[family]``, ``p.launches[family]``."""

    def __enter__(self):
        load().pwd_profile_start()
        return self

    def __exit__(self, *exc):
        n = len(FAMILIES)
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_int * n)()
        load().pwd_profile_stop(ms, cnt, n)
        self.ms = {f: ms[i] for i, f in enumerate(FAMILIES)}
        self.launches = {f: cnt[i] for i, f in enumerate(FAMILIES)}
        return False
