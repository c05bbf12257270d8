"""ctypes front end of the CPU oracle (oracle/pwd_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py``, always as the checker or the timed CPU
baseline, never by the product package.

Each function mirrors the low-level reference entry point it restates
(pyseistr/src/dip_cfuns.c ``dipc``, sof_cfuns.c ``csomean2d``/``csomf2d``,
sof3d_cfuns.c ``csomean3d``/``csomf3d``, soint3d_cfuns.c ``csoint3d``) on
column-major (Fortran-order) float32 or float64 arrays.  ``precision='f32'``
reproduces the reference arithmetic, ``'f64'`` is the FP64 oracle.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "build", "libpwd_oracle.so")
_lib = None

USUM_DOUBLE = 1
FILTER_REAL = 2
TRI_CHUNK = 4
FILTER_FF = 8
TRI_EXACT = 16  # triangle smoothing in double, rounded once per output
GPU_DOTS = 32  # dot products and residual energies in the GPU plain path's summation order
TRUE_RESIDUAL = 512  # precision model: CG residual formed as W x - dat each iteration

_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_long
_F = ctypes.c_float
_D = ctypes.c_double


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (seconds); returns the .so path."""
    src = os.path.join(_HERE, "pwd_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        for pre, R in (("f32", _F), ("f64", _D)):
            getattr(L, f"orc_dip_{pre}").argtypes = [_P, _P, _P] + [_I] * 10 + [_P]
            getattr(L, f"orc_somean2d_{pre}").argtypes = [_P, _P, _P, _I, _I, _I, _I, _I, R, _I]
            getattr(L, f"orc_somf2d_{pre}").argtypes = [_P, _P, _P] + [_I] * 7 + [R]
            getattr(L, f"orc_somean3d_{pre}").argtypes = [_P, _P, _P, _P] + [_I] * 6
            getattr(L, f"orc_somf3d_{pre}").argtypes = [_P, _P, _P, _P] + [_I] * 8
            getattr(L, f"orc_soint3d_{pre}").argtypes = [_P] * 5 + [_I] * 10 + [R]
            getattr(L, f"orc_soint2d_prec_{pre}").argtypes = [_P] * 5 + [_I] * 5
        L.orc_pwspray2d_f32.argtypes = [_P, _P, _P, _I, _I, _I, _I, _F]
        L.orc_pwspray3d_f32.argtypes = [_P, _P, _P, _P] + [_I] * 6
        L.orc_spray_median_f32.argtypes = [_P, _P, _I, _I, _L, _I, _I]
        L.orc_sint2d_f32.argtypes = [_P, _P, _P, _P, _I, _I, _I, _I, _I, _F]
        L.orc_sint3d_f32.argtypes = [_P, _P, _P, _P, _P] + [_I] * 8 + [_F]
        L.orc_paint2d_f32.argtypes = [_P, _P, _P, _I, _I, _I, _I, _F]
        L.orc_coh_f32.argtypes = [_P, _P, _P, _I, _I, _I, _I, _F, _I, _P, _P]
        L.orc_bandpass_f32.argtypes = [_P, _P, _I, _L, _F, _F, _F, _I, _I, _I]
        _lib = L
    return _lib


def _dt(precision):
    if precision not in ("f32", "f64"):
        raise ValueError("precision must be 'f32' or 'f64'")
    return np.float32 if precision == "f32" else np.float64


def _flat(a, dt):
    return np.ascontiguousarray(np.asarray(a, dtype=dt).flatten(order="F"))


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _check(rc, name):
    if rc != 0:
        raise ValueError(f"{name}: invalid arguments (status {rc})")


def dipc(din, n1, n2, n3, niter, liter, order, r1, r2, r3, mask=None, flags=0,
         precision="f32", return_ls=False):
    """Restatement of ``dipc``: returns n (n3==1) or 2n slopes, flat."""
    dt = _dt(precision)
    u = _flat(din, dt)
    n = n1 * n2 * n3
    if u.size != n:
        raise ValueError("data size mismatch")
    m = _flat(mask, dt) if mask is not None else None
    nout = n if n3 == 1 else 2 * n
    out = np.empty(nout, dtype=dt)
    ls = np.zeros(2 * max(niter, 1), dtype=np.int32)
    rc = getattr(lib(), f"orc_dip_{precision}")(
        _ptr(u), _ptr(m), _ptr(out), n1, n2, n3, niter, liter, order, r1, r2, r3, flags, _ptr(ls))
    _check(rc, "dipc")
    return (out, ls) if return_ls else out


def dip2d(din, niter=5, liter=20, order=2, rect=(10, 10, 1), mask=None, flags=0, precision="f32",
          return_ls=False):
    n1, n2 = din.shape
    r = dipc(din, n1, n2, 1, niter, liter, order, rect[0], rect[1], rect[2], mask, flags,
             precision, return_ls)
    if return_ls:
        return r[0].reshape(n1, n2, order="F"), r[1]
    return r.reshape(n1, n2, order="F")


def dip3d(din, niter=5, liter=10, order=2, rect=(5, 5, 5), mask=None, flags=0, precision="f32"):
    n1, n2, n3 = din.shape
    p = dipc(din, n1, n2, n3, niter, liter, order, rect[0], rect[1], rect[2], mask, flags,
             precision)
    p = p.reshape(n1, n2, n3, 2, order="F")
    return p[..., 0], p[..., 1]


def _shape3(dn):
    if dn.ndim == 2:
        return dn.shape[0], dn.shape[1], 1
    return dn.shape


def somean2d(dn, dip, ns, order, eps, adj=0, precision="f32"):
    dt = _dt(precision)
    n1, n2, n3 = _shape3(dn)
    d, p = _flat(dn, dt), _flat(dip, dt)
    out = np.empty(n1 * n2 * n3, dtype=dt)
    rc = getattr(lib(), f"orc_somean2d_{precision}")(_ptr(d), _ptr(p), _ptr(out), n1, n2, n3, ns,
                                                      order, eps, adj)
    _check(rc, "somean2d")
    return out.reshape(dn.shape, order="F")


def somf2d(dn, dip, ns, order, eps, option=1, nmf=None, precision="f32"):
    dt = _dt(precision)
    n1, n2, n3 = _shape3(dn)
    d, p = _flat(dn, dt), _flat(dip, dt)
    out = np.empty(n1 * n2 * n3, dtype=dt)
    nmf = 2 * ns + 1 if nmf is None else nmf
    rc = getattr(lib(), f"orc_somf2d_{precision}")(_ptr(d), _ptr(p), _ptr(out), n1, n2, n3, ns,
                                                    nmf, option, order, eps)
    _check(rc, "somf2d")
    return out.reshape(dn.shape, order="F")


def somean3d(dn, dipi, dipx, r1, r2, order, precision="f32"):
    dt = _dt(precision)
    n1, n2, n3 = _shape3(dn)
    d, p1, p2 = _flat(dn, dt), _flat(dipi, dt), _flat(dipx, dt)
    out = np.empty(n1 * n2 * n3, dtype=dt)
    rc = getattr(lib(), f"orc_somean3d_{precision}")(_ptr(d), _ptr(p1), _ptr(p2), _ptr(out), n1,
                                                      n2, n3, r1, r2, order)
    _check(rc, "somean3d")
    return out.reshape(dn.shape, order="F")


def somf3d(dn, dipi, dipx, r1, r2, order, option=1, nmf=None, precision="f32"):
    dt = _dt(precision)
    n1, n2, n3 = _shape3(dn)
    d, p1, p2 = _flat(dn, dt), _flat(dipi, dt), _flat(dipx, dt)
    out = np.empty(n1 * n2 * n3, dtype=dt)
    nmf = 2 * r1 * r2 + 1 if nmf is None else nmf
    rc = getattr(lib(), f"orc_somf3d_{precision}")(_ptr(d), _ptr(p1), _ptr(p2), _ptr(out), n1,
                                                    n2, n3, r1, r2, nmf, option, order)
    _check(rc, "somf3d")
    return out.reshape(dn.shape, order="F")


def soint3d(din, mask, dipi, dipx, order=1, niter=100, njs=(1, 1), drift=0, seed=202223,
            hasmask=1, var=0.0, precision="f32"):
    dt = _dt(precision)
    n1, n2, n3 = din.shape
    d, m = _flat(din, dt), _flat(mask, dt)
    p, q = _flat(dipi, dt), _flat(dipx, dt)
    out = np.empty(n1 * n2 * n3, dtype=dt)
    rc = getattr(lib(), f"orc_soint3d_{precision}")(
        _ptr(d), _ptr(m), _ptr(p), _ptr(q), _ptr(out), n1, n2, n3, order, njs[0], njs[1], niter,
        drift, seed, hasmask, var)
    _check(rc, "soint3d")
    return out.reshape(n1, n2, n3, order="F")


def soint2d_prec(din, mask, dip, order=1, niter=100, hasmask=1, twoplane=0, precision="f32"):
    """csoint2d with prec = 1: dip is [n1, n2] (one plane) or [n1, n2, 2]
    (twoplane, the two planes' slopes)."""
    dt = _dt(precision)
    n1, n2 = din.shape[:2]
    d, m = _flat(din, dt), _flat(mask, dt)
    if twoplane:
        p, q = _flat(dip[:, :, 0], dt), _flat(dip[:, :, 1], dt)
    else:
        p, q = _flat(dip, dt), None
    out = np.empty(n1 * n2, dtype=dt)
    rc = getattr(lib(), f"orc_soint2d_prec_{precision}")(
        _ptr(d), _ptr(m), _ptr(p), _ptr(q) if q is not None else None, _ptr(out), n1, n2, order,
        niter, hasmask)
    _check(rc, "soint2d_prec")
    return out.reshape(n1, n2, order="F")


def pwspray2d(dn, dip, ns, order, eps):
    """Sprayed panels u[n2][2ns+1][n1] (C order) of one 2-D section."""
    n1, n2 = dn.shape
    d, p = _flat(dn, np.float32), _flat(dip, np.float32)
    u = np.empty((n2, 2 * ns + 1, n1), dtype=np.float32)
    _check(lib().orc_pwspray2d_f32(_ptr(d), _ptr(p), _ptr(u), n1, n2, ns, order, eps), "pwspray2d")
    return u


def pwspray3d(dn, dipi, dipx, r1, r2, order):
    """Sprayed panels u[n2*n3][np][n1] (C order) of one 3-D cube."""
    n1, n2, n3 = dn.shape
    npp = (2 * r1 + 1) * (2 * r2 + 1)
    d, p1, p2 = (_flat(a, np.float32) for a in (dn, dipi, dipx))
    u = np.empty((n2 * n3, npp, n1), dtype=np.float32)
    _check(lib().orc_pwspray3d_f32(_ptr(d), _ptr(p1), _ptr(p2), _ptr(u), n1, n2, n3, r1, r2, order),
           "pwspray3d")
    return u


def spray_median(u, nmf, option=1):
    """Median row (np-1)/2 of sprayed panels u[ntr][np][n1] -> out[ntr][n1]."""
    u = np.ascontiguousarray(u, dtype=np.float32)
    ntr, npp, n1 = u.shape
    out = np.empty((ntr, n1), dtype=np.float32)
    _check(lib().orc_spray_median_f32(_ptr(u), _ptr(out), n1, npp, ntr, nmf, option), "median")
    return out


def bandpass(din, dt, flo=0.0, fhi=0.5, nplo=6, nphi=6, phase=0):
    """cbp (pyseistr/src/bp_cfuns.c:524-645): Butterworth band-pass of every
    trace of a column-major (n1, n2[, n3]) float32 array; same shape out."""
    a = np.asarray(din, dtype=np.float32)
    n1 = a.shape[0]
    ntr = a.size // n1
    x = _flat(a, np.float32)
    out = np.empty_like(x)
    _check(lib().orc_bandpass_f32(_ptr(x), _ptr(out), n1, ntr, dt, flo, fhi, nplo, nphi,
                                  phase), "bandpass")
    return out.reshape(a.shape, order="F")



def sint2d(din, mask, dip, niter=100, eps=0.01, ns=1, order=1):
    """csint2d (pyseistr/src/soint2d_cfuns.c:2421-2523): sparse-data
    interpolation of an (n1, n2) section, known samples where mask != 0."""
    a = np.asarray(din, dtype=np.float32)
    n1, n2 = a.shape
    d, m, p = _flat(a, np.float32), _flat(mask, np.float32), _flat(dip, np.float32)
    out = np.empty_like(d)
    _check(lib().orc_sint2d_f32(_ptr(d), _ptr(p), _ptr(m), _ptr(out), n1, n2, niter, ns, order,
                                eps), "sint2d")
    return out.reshape(n1, n2, order="F")


def sint3d(din, mask, dipi, dipx, niter=100, eps=0.01, ns1=1, ns2=1, order1=1, order2=1):
    """csint3d (pyseistr/src/soint3d_cfuns.c:2510-2612): sparse-data
    interpolation of an (n1, n2, n3) cube, known samples where mask != 0."""
    a = np.asarray(din, dtype=np.float32)
    n1, n2, n3 = a.shape
    d, m = _flat(a, np.float32), _flat(mask, np.float32)
    p, q = _flat(dipi, np.float32), _flat(dipx, np.float32)
    out = np.empty_like(d)
    _check(lib().orc_sint3d_f32(_ptr(d), _ptr(p), _ptr(q), _ptr(m), _ptr(out), n1, n2, n3, niter,
                                ns1, ns2, order1, order2, eps), "sint3d")
    return out.reshape(n1, n2, n3, order="F")


def paint2d(dip, seed, order=1, i0=0, eps=0.01):
    """cpaint2d (pyseistr/src/paint_cfuns.c:1861-1940): plane-wave painting
    of the seed trace from trace i0 along the slope dip (n1, n2)."""
    p = np.asarray(dip, dtype=np.float32)
    n1, n2 = p.shape
    t = _flat(seed, np.float32)
    if t.size != n1:
        raise ValueError(f"paint2d: the seed trace has {t.size} samples, expected {n1}")
    out = np.empty(n1 * n2, dtype=np.float32)
    _check(lib().orc_paint2d_f32(_ptr(_flat(p, np.float32)), _ptr(t), _ptr(out), n1, n2, order,
                                 i0, eps), "paint2d")
    return out.reshape(n1, n2, order="F")


class Coherence:
    """cohc_fb (pyseistr/src/coh_cfuns.c:415-545): forward (forw 1: model
    [nt, nv] -> data [nt, nh]) and adjoint coherence (forw -1: data ->
    model) Radon operators.  Keeps the parabolic type's hmax across calls,
    as the reference's file-scope static does within one process."""

    def __init__(self):
        self.hmax = np.zeros(1, dtype=np.float32)

    def __call__(self, din, v, h, typ, nt, dt, forw):
        v = np.ascontiguousarray(v, dtype=np.float32)
        h = np.ascontiguousarray(h, dtype=np.float32)
        nv, nh = v.size, h.size
        x = _flat(din, np.float32)
        out = np.empty(nt * (nh if forw == 1 else nv), dtype=np.float32)
        _check(lib().orc_coh_f32(_ptr(x), _ptr(v), _ptr(h), typ, nt, nv, nh, dt, forw, _ptr(out),
                                 _ptr(self.hmax)), "coh")
        return out.reshape(nt, -1, order="F")
