"""pyseistr-compatible host API on the GB300 kernels.

Same names, signatures, defaults and return types as the reference's C-path
wrappers (pyseistr/dip2d.py:115 dip2dc, dip3d.py:59 dip3dc,
somean2d.py:36 somean2dc, somf2d.py:60 somf2dc, somean3d.py:36 somean3dc,
somf3d.py:54 somf3dc, soint3d.py:65 soint3dc) and low-level entries (dipc,
csomean2d, csomf2d, csomean3d, csomf3d, csoint3d with the reference's
positional argument tuples).  NumPy inputs are flattened in Fortran order to
float32, copied to the GPU, processed and copied back as NumPy float32;
CUDA tensors stay on the device and CUDA tensors are returned.

Arguments the reference C ignores are accepted and ignored here too
(eps_dv, eps_cg, tol_cg of dip*; eps of the 3-D filters is replaced by 0.01;
verb, runc).  Bad sizes raise ValueError where the reference prints
"Dimension mismatch" and returns NULL.
"""
from __future__ import annotations

import numpy as np
import torch

from . import device as D


_COPY_STREAMS = {}


def _copy_stream():
    """A side stream of the current device for device-to-host copies that
    overlap later kernels."""
    dev = torch.cuda.current_device()
    if dev not in _COPY_STREAMS:
        _COPY_STREAMS[dev] = torch.cuda.Stream(device=dev)
    return _COPY_STREAMS[dev]


def _dev():
    if not torch.cuda.is_available():
        raise RuntimeError("pyseistr_gb300 needs a CUDA GPU; no CPU fallback exists")
    return torch.device("cuda", torch.cuda.current_device())


def _to_dev_flat(a):
    """(array, was_tensor): a flat float32 CUDA tensor in Fortran order."""
    if isinstance(a, torch.Tensor):
        t = a.to(device=_dev(), dtype=torch.float32)
        t = t.permute(*reversed(range(t.dim()))).contiguous().view(-1)
        return t, True
    arr = np.asarray(a, dtype=np.float32)
    flat = np.ascontiguousarray(arr.reshape(-1, order="F"))
    pinned = torch.from_numpy(flat).pin_memory()
    return pinned.to(_dev(), non_blocking=True), False


def _from_dev_flat(t, shape, as_tensor):
    if as_tensor:
        return t.view(*reversed(shape)).permute(*reversed(range(len(shape))))
    host = t.cpu().numpy()
    return host.reshape(shape, order="F")


# --------------------------------------------------------------------------
# low-level entries (reference positional tuples)
# --------------------------------------------------------------------------
def dipc(din, n1, n2, n3, niter, liter, order, eps_dv, eps_cg, tol_cg, r1, r2, r3, hasmask,
         verb):
    """dipc "Oiiiiiifffiiiii" (dip_cfuns.c:1708): din is [data] or [data, mask]."""
    t, as_t = _to_dev_flat(din)
    n = n1 * n2 * n3
    if hasmask:
        if t.numel() != 2 * n:
            raise ValueError(f"Dimension mismatch, N_input = {t.numel()}, N_data = {2 * n}")
        data, mask = t[:n], t[n:]
    else:
        if t.numel() != n:
            raise ValueError(f"Dimension mismatch, N_input = {t.numel()}, N_data = {n}")
        data, mask = t, None
    out = D.dip(data, n1, n2, n3, niter, liter, order, (r1, r2, r3), mask)
    return out if as_t else out.cpu().numpy()


def csomean2d(dn, dip, n1, n2, n3, ns, order, adj, eps, verb):
    d, as_t = _to_dev_flat(dn)
    p, _ = _to_dev_flat(dip)
    out = D.somean2d(d, p, n1, n2, n3, ns, order, eps, adj)
    return out if as_t else out.cpu().numpy()


def csomf2d(dn, dip, n1, n2, n3, ns, nmf, option, order, eps, verb):
    d, as_t = _to_dev_flat(dn)
    p, _ = _to_dev_flat(dip)
    out = D.somf2d(d, p, n1, n2, n3, ns, nmf, option, order, eps)
    return out if as_t else out.cpu().numpy()


def csomean3d(dn, dipi, dipx, n1, n2, n3, r1, r2, order, eps, verb):
    d, as_t = _to_dev_flat(dn)
    pi, _ = _to_dev_flat(dipi)
    px, _ = _to_dev_flat(dipx)
    out = D.somean3d(d, pi, px, n1, n2, n3, r1, r2, order, eps)
    return out if as_t else out.cpu().numpy()


def csomf3d(dn, dipi, dipx, n1, n2, n3, r1, r2, nmf, option, order, eps, verb):
    d, as_t = _to_dev_flat(dn)
    pi, _ = _to_dev_flat(dipi)
    px, _ = _to_dev_flat(dipx)
    out = D.somf3d(d, pi, px, n1, n2, n3, r1, r2, nmf, option, order, eps)
    return out if as_t else out.cpu().numpy()


def csoint3d(din, mask, dipi, dipx, n1, n2, n3, nw, nj1, nj2, niter, drift, seed, hasmask, var,
             verb):
    d, as_t = _to_dev_flat(din)
    m, _ = _to_dev_flat(mask)
    pi, _ = _to_dev_flat(dipi)
    px, _ = _to_dev_flat(dipx)
    out = D.soint3d(d, m, pi, px, n1, n2, n3, nw, nj1, nj2, niter, drift, seed, hasmask, var)
    return out if as_t else out.cpu().numpy()


def csoint2d(din, mask, dip1, dip2, n1, n2, nw, nj1, nj2, niter, drift, hasmask, twoplane, prec,
             verb):
    """csoint2d "OOOOiiiiiiiiiii" (soint2d_cfuns.c:2260).  Its default branch
    (twoplane 0, prec 0: allpass21_lop inside ps_solver with the known mask
    and x0) is csoint3d's operator and solver with n3 = 1 (the crossline
    rows are empty), computed here by pwd_soint3d; the two-plane branch
    without preconditioning returns din unchanged, as the reference's (its
    solver call is commented out).  The preconditioned branches (prec 1:
    ps_solver_prec with predict_lop along dip1, or predict2_lop chaining dip1
    and dip2 when twoplane) run in pwd_soint2d_prec."""
    n = n1 * n2
    d, as_t = _to_dev_flat(din)
    if d.numel() != n:
        raise ValueError(f"csoint2d: din has {d.numel()} values, expected {n}")
    if prec:
        m, _ = _to_dev_flat(mask)
        p1, _ = _to_dev_flat(dip1)
        p2 = _to_dev_flat(dip2)[0] if twoplane else None
        out = D.soint2d_prec(d, m, p1, p2, n1, n2, nw, niter, hasmask, twoplane)
    elif twoplane:
        out = d.clone()
    else:
        m, _ = _to_dev_flat(mask)
        p, _ = _to_dev_flat(dip1)
        out = D.soint3d(d, m, p, p, n1, n2, 1, nw, nj1, nj2, niter, drift, 202223, hasmask, 0.0)
    return out if as_t else out.cpu().numpy()


# --------------------------------------------------------------------------
# high-level entries
# --------------------------------------------------------------------------
def dip2dc(din, niter=5, liter=20, order=2, eps_dv=0.01, eps_cg=1, tol_cg=0.000001,
           rect=[10, 10, 1], verb=1, mask=None, mixed=False):
    """2-D slope by shaping-regularised PWD (dip2d.py:115).  mixed=True (not
    in the reference) estimates it in the mixed mode: FP32 taps, the
    smoothing as a fused direct convolution, FP64 reductions; about 1e-7
    from an FP64 evaluation instead of the reference's bits."""
    n1, n2 = din.shape[0], din.shape[1]
    d, as_t = _to_dev_flat(din)
    m = None
    if mask is not None:
        if int(np.prod(mask.shape)) != n1 * n2:
            raise ValueError("Mask and Data should have the same dimension")
        m, _ = _to_dev_flat(mask)
    if mixed:
        out = D.dip_batch(d, [(n1, n2)], niter, liter, order, rect, mask=m, mixed=True)
    else:
        out = D.dip(d, n1, n2, 1, niter, liter, order, rect, m)
    return _from_dev_flat(out, (n1, n2), as_t)


def dip3dc(din, niter=5, liter=10, order=2, eps_dv=0.01, eps_cg=1, tol_cg=0.000001,
           rect=[5, 5, 5], verb=1, runc=1, mask=None, mixed=False):
    """3-D inline and crossline slopes (dip3d.py:59); mixed=True as in
    dip2dc."""
    n1, n2, n3 = din.shape
    d, as_t = _to_dev_flat(din)
    m = None
    if mask is not None:
        if int(np.prod(mask.shape)) != n1 * n2 * n3:
            raise ValueError("Mask and Data should have the same dimension")
        m, _ = _to_dev_flat(mask)
    if mixed:
        out = D.dip_batch(d, [(n1, n2, n3)], niter, liter, order, rect, mask=m, mixed=True)
    else:
        out = D.dip(d, n1, n2, n3, niter, liter, order, rect, m)
    n = n1 * n2 * n3
    return (_from_dev_flat(out[:n], (n1, n2, n3), as_t),
            _from_dev_flat(out[n:], (n1, n2, n3), as_t))


def _shape3(dn):
    if dn.ndim == 2:
        return dn.shape[0], dn.shape[1], 1
    return tuple(dn.shape)


def somean2dc(dn, dip, ns, order, eps, adj=0, verb=1):
    """Structure-oriented (triangle-weighted) mean, 2-D slices (somean2d.py:36)."""
    n1, n2, n3 = _shape3(dn)
    d, as_t = _to_dev_flat(dn)
    p, _ = _to_dev_flat(dip)
    out = D.somean2d(d, p, n1, n2, n3, ns, order, eps, adj)
    res = _from_dev_flat(out, (n1, n2, n3), as_t)
    return res.squeeze() if n3 == 1 else res


def somf2dc(dn, dip, ns, order, eps, option=1, verb=1):
    """Structure-oriented median filter, 2-D slices (somf2d.py:60)."""
    n1, n2, n3 = _shape3(dn)
    d, as_t = _to_dev_flat(dn)
    p, _ = _to_dev_flat(dip)
    out = D.somf2d(d, p, n1, n2, n3, ns, 2 * ns + 1, option, order, eps)
    res = _from_dev_flat(out, (n1, n2, n3), as_t)
    return res.squeeze() if n3 == 1 else res


def somean3dc(dn, dipi, dipx, r1, r2, eps, order, verb=0):
    """3-D structure-oriented mean (somean3d.py:36)."""
    n1, n2, n3 = _shape3(dn)
    d, as_t = _to_dev_flat(dn)
    pi, _ = _to_dev_flat(dipi)
    px, _ = _to_dev_flat(dipx)
    out = D.somean3d(d, pi, px, n1, n2, n3, r1, r2, order, eps)
    return _from_dev_flat(out, (n1, n2, n3), as_t)


def somf3dc(dn, dipi, dipx, r1, r2, eps, order, option=1, verb=1):
    """3-D structure-oriented median filter (somf3d.py:54)."""
    n1, n2, n3 = _shape3(dn)
    d, as_t = _to_dev_flat(dn)
    pi, _ = _to_dev_flat(dipi)
    px, _ = _to_dev_flat(dipx)
    out = D.somf3d(d, pi, px, n1, n2, n3, r1, r2, 2 * r1 * r2 + 1, option, order, eps)
    return _from_dev_flat(out, (n1, n2, n3), as_t)


def soint3dc(din, mask, dipi, dipx, order=1, niter=100, njs=[1, 1], drift=0, seed=202223,
             hasmask=1, var=0, verb=1):
    """3-D structure-oriented interpolation (soint3d.py:65)."""
    n1, n2, n3 = din.shape
    d, as_t = _to_dev_flat(din)
    m, _ = _to_dev_flat(mask)
    pi, _ = _to_dev_flat(dipi)
    px, _ = _to_dev_flat(dipx)
    out = D.soint3d(d, m, pi, px, n1, n2, n3, order, njs[0], njs[1], niter, drift, seed, hasmask,
                    var)
    return _from_dev_flat(out, (n1, n2, n3), as_t)


def soint2dc(din, mask, dip, order=1, niter=100, njs=[1, 1], drift=0, hasmask=1, twoplane=0,
             prec=0, verb=1):
    """2-D structure-oriented interpolation (soint2d.py:92): fills the
    samples the mask marks unknown (mask 0, or din 0 when hasmask is 0) by
    conjugate gradients on the plane-wave-destruction residual along the
    slope field dip [n1, n2] (the first plane of a [n1, n2, 2] dip when
    twoplane).  order = PWD accuracy order, njs = antialiasing steps, drift
    = shift the filter by the rounded slope."""
    n1, n2 = din.shape[:2]
    dip1 = dip if twoplane == 0 else dip[:, :, 0]
    d, as_t = _to_dev_flat(din)
    if prec:
        # soint2d_cfuns.c:2354-2398: CG on M P p = d with the plane-wave
        # integration P (predict_lop, or predict2_lop chaining both planes)
        m, _ = _to_dev_flat(mask)
        p1, _ = _to_dev_flat(dip1)
        p2 = _to_dev_flat(dip[:, :, 1])[0] if twoplane else None
        out = D.soint2d_prec(d, m, p1, p2, n1, n2, order, niter, hasmask, twoplane)
        return _from_dev_flat(out, (n1, n2), as_t)
    if twoplane:
        # the reference's two-plane branch without preconditioning runs no
        # solver and returns the data unchanged
        return _from_dev_flat(d.clone(), (n1, n2), as_t)
    m, _ = _to_dev_flat(mask)
    p, _ = _to_dev_flat(dip1)
    out = D.soint3d(d, m, p, p, n1, n2, 1, order, njs[0], njs[1], niter, drift, 202223, hasmask,
                    0.0)
    return _from_dev_flat(out, (n1, n2), as_t)


# --------------------------------------------------------------------------
# batched entries: many sections of uneven size in one launch sequence
# --------------------------------------------------------------------------
def _pack(sections):
    flat = np.concatenate([np.asarray(s, np.float32).reshape(-1, order="F") for s in sections])
    t = torch.from_numpy(flat).pin_memory().to(_dev(), non_blocking=True)
    return t


def _unpack(t, shapes):
    host = t.cpu().numpy()
    out, k = [], 0
    for sh in shapes:
        n = int(np.prod(sh))
        out.append(host[k:k + n].reshape(sh, order="F"))
        k += n
    return out


def dip_somean2d_packed(data, shapes, niter=5, liter=10, order=2, rect=[10, 10, 1], ns=6,
                        eps=0.01, median=False, mixed=False, out=None):
    """dip_somean2d_batch on sections already packed one after another in a
    flat float32 tensor (each section column-major): a CPU tensor, pinned
    for full-speed copies, or a CUDA tensor.  Returns (slopes, filtered) as
    flat CPU tensors (pinned), or fills `out` = (slopes, filtered) when
    given.  One host-to-device copy in, two device-to-host copies out."""
    if not isinstance(data, torch.Tensor) or data.dtype != torch.float32 or data.dim() != 1:
        raise TypeError("data must be a flat float32 tensor")
    d = data if data.is_cuda else data.to(_dev(), non_blocking=True)
    p = D.dip_batch(d, shapes, niter, liter, order, rect, mixed=mixed)
    if out is None:
        out = (torch.empty(p.shape, dtype=torch.float32, pin_memory=True),
               torch.empty(d.shape, dtype=torch.float32, pin_memory=True))
    # the slopes go down on a side stream while the filter runs
    cur = torch.cuda.current_stream()
    side = _copy_stream()
    side.wait_stream(cur)
    with torch.cuda.stream(side):
        out[0].copy_(p, non_blocking=True)
    p.record_stream(side)
    f = D.sofilter2d_batch(d, p, shapes, ns, order, eps,
                           filter=D.FILTER_MEDIAN if median else D.FILTER_MEAN)
    out[1].copy_(f, non_blocking=True)
    cur.synchronize()
    side.synchronize()
    return out


def dip_soint3d_packed(data, mask, shapes, niter=5, liter=10, order=2, rect=[5, 5, 5],
                       soint_order=2, soint_niter=20, mixed=False, out=None):
    """Slopes of many cubes (dip3dc on each) followed by their interpolation
    (soint3dc with the cube's mask, order soint_order, niter soint_niter),
    on cubes packed one after another in flat float32 tensors `data` and
    `mask` (CPU, pinned for full-speed copies, or CUDA).  The slopes are
    estimated on data as given; the interpolation sees data * mask.
    Returns the interpolated cubes as one flat CPU tensor (pinned), or fills
    `out`.  One copy of data and mask in, one copy out."""
    for t, name in ((data, "data"), (mask, "mask")):
        if not isinstance(t, torch.Tensor) or t.dtype != torch.float32 or t.dim() != 1:
            raise TypeError(f"{name} must be a flat float32 tensor")
    d = data if data.is_cuda else data.to(_dev(), non_blocking=True)
    m = mask if mask.is_cuda else mask.to(_dev(), non_blocking=True)
    p = D.dip_batch(d, shapes, niter, liter, order, rect, mixed=mixed)
    x = D.soint3d_batch(d * m, m, p, shapes, order=soint_order, niter=soint_niter)
    if out is None:
        out = torch.empty(x.shape, dtype=torch.float32, pin_memory=True)
    out.copy_(x, non_blocking=True)
    torch.cuda.current_stream().synchronize()
    return out


def dip2dc_batch(sections, niter=5, liter=20, order=2, rect=[10, 10, 1], mixed=False):
    """dip2dc over a list of 2-D sections, all in one launch sequence;
    returns the list of slopes (each equal to dip2dc of its section, or its
    mixed-mode approximation with mixed=True)."""
    shapes = [tuple(s.shape) for s in sections]
    out = D.dip_batch(_pack(sections), shapes, niter, liter, order, rect, mixed=mixed)
    return _unpack(out, shapes)


def somean2dc_batch(sections, dips, ns, order, eps, adj=0):
    """somean2dc over a list of 2-D sections and their slopes."""
    shapes = [tuple(s.shape) for s in sections]
    out = D.sofilter2d_batch(_pack(sections), _pack(dips), shapes, ns, order, eps,
                             filter=D.FILTER_MEAN_ADJ if adj else D.FILTER_MEAN)
    return _unpack(out, shapes)


def somf2dc_batch(sections, dips, ns, order, eps, option=1):
    """somf2dc over a list of 2-D sections and their slopes."""
    shapes = [tuple(s.shape) for s in sections]
    out = D.sofilter2d_batch(_pack(sections), _pack(dips), shapes, ns, order, eps,
                             filter=D.FILTER_MEDIAN, nmf=2 * ns + 1, option=option)
    return _unpack(out, shapes)


def soint2dc_batch(sections, masks, dips, order=1, niter=100, hasmask=1, twoplane=0):
    """soint2dc(..., prec=1) over a list of 2-D sections, their masks and
    slopes ([n1, n2], or [n1, n2, 2] when twoplane), one CTA per section;
    returns the list of results (each equal to its own call's)."""
    shapes = [tuple(s.shape[:2]) for s in sections]
    d1 = [d if not twoplane else d[:, :, 0] for d in dips]
    d2 = _pack([d[:, :, 1] for d in dips]) if twoplane else None
    out = D.soint2d_prec_batch(_pack(sections), _pack(masks), _pack(d1), d2, shapes, order,
                               niter, hasmask, twoplane)
    return _unpack(out, shapes)


def dip_somean2d_batch(sections, niter=5, liter=10, order=2, rect=[10, 10, 1], ns=6, eps=0.01,
                       median=False, mixed=False):
    """Slope estimation followed by the structure-oriented mean (or median)
    of many sections: one upload, both stages on the device, one download.
    Returns (slopes, filtered) lists.  mixed=True estimates the slopes in
    the mixed mode."""
    shapes = [tuple(s.shape) for s in sections]
    d = _pack(sections)
    p = D.dip_batch(d, shapes, niter, liter, order, rect, mixed=mixed)
    if median:
        f = D.sofilter2d_batch(d, p, shapes, ns, order, eps, filter=D.FILTER_MEDIAN)
    else:
        f = D.sofilter2d_batch(d, p, shapes, ns, order, eps, filter=D.FILTER_MEAN)
    return _unpack(p, shapes), _unpack(f, shapes)


def _mode1(mode):
    if mode != 1:
        raise ValueError("patching mode 1 is the only mode the reference defines")


def _patches_to_dev(X, npatch, m):
    """The patch matrix (rows = patches) as a flat CUDA tensor, row-major."""
    if isinstance(X, torch.Tensor):
        t = X.to(device=_dev(), dtype=torch.float32).reshape(-1).contiguous()
        return t, True
    arr = np.ascontiguousarray(np.asarray(X, dtype=np.float32).reshape(npatch, m))
    return torch.from_numpy(arr.reshape(-1)).pin_memory().to(_dev(), non_blocking=True), False


def _patch_fwd(A, ls, ss):
    shape = tuple(A.shape)
    a, as_t = _to_dev_flat(A)
    x = D.patch(a, shape, ls, ss)
    return x if as_t else x.cpu().numpy()


def _patch_inv(X, shape, ls, ss):
    npatch = D.patch_count(shape, ls, ss)
    if npatch == 0:
        raise ValueError("invalid patch sizes")
    m = int(np.prod(ls))
    x, as_t = _patches_to_dev(X, npatch, m)
    out = D.patch_inv(x, shape, ls, ss)
    return _from_dev_flat(out, shape, as_t)


def patch2d(A, l1=8, l2=8, s1=4, s2=4, mode=1):
    """patch2d (patch.py:2): the l1 x l2 windows of a 2-D array at strides
    s1, s2 (the array zero-padded at its ends so that the last window ends
    on it) as the rows of a [npatch, l1*l2] float32 array, each window
    flattened column-major; rows are ordered with the first axis's window
    starts outermost.  A CUDA tensor in gives a CUDA tensor out."""
    _mode1(mode)
    return _patch_fwd(A, (l1, l2), (s1, s2))


def patch3d(A, l1=4, l2=4, l3=4, s1=2, s2=2, s3=2, mode=1):
    """patch3d (patch.py:86): as patch2d for a 3-D array; the result has the
    reference's trailing axis of length 1, [npatch, l1*l2*l3, 1]."""
    _mode1(mode)
    x = _patch_fwd(A, (l1, l2, l3), (s1, s2, s3))
    return x.unsqueeze(-1) if isinstance(x, torch.Tensor) else x[:, :, None]


def patch2d_inv(X, n1, n2, l1=8, l2=8, s1=4, s2=4, mode=1):
    """patch2d_inv (patch.py:208): overlap-add of the patches into an n1 x n2
    float32 array, each sample divided by the number of windows covering it
    (NaN where none does)."""
    _mode1(mode)
    return _patch_inv(X, (n1, n2), (l1, l2), (s1, s2))


def patch3d_inv(X, n1, n2, n3, l1=4, l2=4, l3=4, s1=2, s2=2, s3=2, mode=1):
    """patch3d_inv (patch.py:307): as patch2d_inv for 3-D, from [npatch, L]
    or the [npatch, L, 1] that patch3d returns.  Every pattern of padded
    axes is handled (the reference's leaves two of them unassigned and
    raises)."""
    _mode1(mode)
    return _patch_inv(X, (n1, n2, n3), (l1, l2, l3), (s1, s2, s3))


# --------------------------------------------------------------------------
# band-pass (bp.py / bp_cfuns.c)
# --------------------------------------------------------------------------
def _bp_messages(n123, dt, flo, fhi, nplo, nphi, phase, verb):
    """cbp's console output (bp_cfuns.c:544-580): the range warnings always,
    the parameter lines when verb."""
    f32 = np.float32
    if verb:
        print("nplo=%d,n123=%d" % (nplo, n123))
    flo, fhi = f32(flo), f32(fhi)
    if flo < 0:
        print("Negative flo", end="")
    else:
        flo = f32(flo * f32(dt))
    if fhi < 0:
        print("Negative flo", end="")
    else:
        fhi = f32(fhi * f32(dt))
        if flo > fhi:
            print("Need flo < fhi")
        if 0.5 < fhi:
            print("Need fhi < Nyquist")
    if verb:
        nlo = max(int(nplo), 1)
        nhi = max(int(nphi), 1)
        nlo = nlo // 2 if nlo > 1 and not phase else nlo
        nhi = nhi // 2 if nhi > 1 and not phase else nhi
        print("flo=%g fhi=%g nplo=%d nphi=%d" % (float(flo), float(fhi), nlo, nhi))


def cbp(din, n1, n2, n3, dt, flo, fhi, nplo, nphi, phase, verb):
    """cbp "Oiiifffiiii" (bp_cfuns.c:524): Butterworth band-pass of the n2*n3
    traces of length n1 in the flat column-major din; returns the flat
    float32 result (a CUDA tensor for a tensor in)."""
    t, as_t = _to_dev_flat(din)
    n = n1 * n2 * n3
    if t.numel() != n:
        raise ValueError(f"cbp: din has {t.numel()} values, expected {n}")
    _bp_messages(n, dt, flo, fhi, nplo, nphi, phase, verb)
    out = D.bandpass(t, (n1, n2, n3), dt, flo, fhi, nplo, nphi, phase)
    return out if as_t else out.cpu().numpy()


def bandpassc(din, dt, flo=0, fhi=0.5, nplo=6, nphi=6, phase=0, verb=1):
    """bandpassc (bp.py:128): Butterworth band-pass along the first axis.
    flo, fhi in Hz (dt in s); a cut-off of 0 (low) or at or above Nyquist
    (high) is not applied; nplo, nphi poles (halved for zero phase); phase
    0 = zero phase (each filter forward, then backward), 1 = minimum phase.
    1-D, 2-D or 3-D float32 in, same shape out, squeezed when the third
    axis has length 1; a CUDA tensor in gives a CUDA tensor out."""
    shape = tuple(din.shape)
    if len(shape) == 1:
        shape = (shape[0], 1, 1)
    elif len(shape) == 2:
        shape = (shape[0], shape[1], 1)
    elif len(shape) != 3:
        raise ValueError("bandpassc: din must have 1, 2 or 3 axes")
    if shape[0] == 1 and shape[1] > 1 and shape[2] == 1:
        # the reference flattens a row vector and then fails to unpack its shape
        raise ValueError("bandpassc: a 1 x n row vector is not accepted (the reference raises)")
    n1, n2, n3 = shape
    if n1 * n2 * n3 == 0:
        raise ValueError("bandpassc: empty input")
    t, as_t = _to_dev_flat(din)
    _bp_messages(n1 * n2 * n3, dt, flo, fhi, nplo, nphi, phase, verb)
    out = D.bandpass(t, shape, dt, flo, fhi, nplo, nphi, phase)
    dout = _from_dev_flat(out, shape, as_t)
    if n3 == 1:
        dout = dout.squeeze() if as_t else np.squeeze(dout)
    return dout


# --------------------------------------------------------------------------
# Radon coherence (das.py cohc / coh_cfuns.c cohc_fb)
# --------------------------------------------------------------------------
class _CohState:
    """The parabolic normaliser hmax, which the reference keeps in a
    file-scope static of coh_cfuns.c for the life of the process: it starts
    at 0 and coh_init2 (coh_cfuns.c:158-179) updates it from every parabolic
    call's offsets (to the signed offset h[i] whenever hmax < |h[i]|)."""

    def __init__(self):
        self.hmax = np.float32(0.0)

    def update(self, h):
        hm = float(self.hmax)
        for x in h.tolist():
            if hm < abs(x):
                hm = x
        self.hmax = np.float32(hm)


coh_state = _CohState()


def _coh_indices_usable(v, h, typ, nt, dt, hmax):
    """Whether every curve's sample index floor(t / dt) + 1 is a finite value
    below 2e9 in magnitude, evaluated in float32 as the kernels do.  The
    index is monotone along each curve (in itau), so its two ends decide."""
    f32 = np.float32
    dt = f32(dt)
    hh, vv = h[:, None], v[None, :]
    with np.errstate(all="ignore"):
        for itau in (0, nt - 1):
            if typ == 2:
                t = f32(itau) * dt + hh * hh * vv / hmax / hmax
            elif typ == 3:
                tau = f32(itau) * dt
                hv = hh / vv
                t = np.sqrt(tau * tau + hv * hv)
            else:
                t = f32(itau) * dt + hh * vv
            fl = np.floor(t / dt) + f32(1)
            if not (np.abs(fl) < f32(2.0e9)).all():
                return False
    return True


def _host_f32(a, name):
    if isinstance(a, torch.Tensor):
        a = a.detach().cpu().numpy()
    a = np.asarray(a, dtype=np.float32).reshape(-1)
    return np.ascontiguousarray(a)


def cohc_fb(din, v, h, typ, nt, nv, nh, dt, forw, verb):
    """cohc_fb "OOOiiiifii" (coh_cfuns.c:415): forw = 1 maps the flat model
    [nv][nt] to the flat data [nh][nt], forw = -1 the data to the coherence
    model num^2 / (nh den + 1e-16); typ 1 linear, 2 parabolic, 3 hyperbolic
    (others linear).  Returns a flat float32 array (a CUDA tensor for a
    tensor in).  A curve reaching past the end of the data (sample nt of the
    last trace), where the reference reads whatever follows its array, reads
    0 there.  Raises ValueError for forw other
    than 1 or -1, for fewer values than the sizes name (the reference reads
    past its arrays), and for curves with no usable sample index (NaN, or
    2e9 samples or more; the reference's int conversion is undefined)."""
    typ, nt, nv, nh, forw = int(typ), int(nt), int(nv), int(nh), int(forw)
    if verb:
        print("typ=%d,nt0=%d,nv0=%d,nh0=%d,dt0=%g,forw=%d,verb=%d"
              % (typ, nt, nv, nh, float(np.float32(dt)), forw, verb))
    if forw not in (1, -1):
        raise ValueError(f"cohc_fb: forw must be 1 or -1, got {forw}")
    if nt < 1 or nv < 1 or nh < 1:
        raise ValueError("cohc_fb: nt, nv and nh must be positive")
    vh, hh = _host_f32(v, "v"), _host_f32(h, "h")
    if vh.size < nv or hh.size < nh:
        raise ValueError(f"cohc_fb: {vh.size} velocities and {hh.size} offsets, expected "
                         f"{nv} and {nh}")
    vh, hh = vh[:nv].copy(), hh[:nh].copy()
    if typ not in (1, 2, 3):
        typ = 1
    if typ == 2:
        coh_state.update(hh)
    if not _coh_indices_usable(vh, hh, typ, nt, dt, coh_state.hmax):
        raise ValueError("cohc_fb: curve sample indices not finite or beyond 2e9 samples")
    t, as_t = _to_dev_flat(din)
    need = nt * (nv if forw == 1 else nh)
    if t.numel() < need:
        raise ValueError(f"cohc_fb: din has {t.numel()} values, expected {need}")
    t = t[:need].contiguous()
    dev = t.device
    vt = torch.from_numpy(vh).to(dev)
    ht = torch.from_numpy(hh).to(dev)
    out = D.coherence(t, vt, ht, typ, nt, dt, forw, coh_state.hmax)
    return out if as_t else out.cpu().numpy()


def cohc(din, par, operator=-1, verb=0):
    """cohc (das.py:92): time-domain Radon coherence.  par holds 'h'
    (offsets), 'v' (curve parameters), 'nt', 'dt' and 'typ'; operator 1 is
    the forward map of an (nt, nv) model to (nt, nh) data, -1 (the default)
    the coherence of (nt, nh) data as an (nt, nv) model; a CUDA tensor in
    gives a CUDA tensor out."""
    h, v = _host_f32(par["h"], "h"), _host_f32(par["v"], "v")
    nt, dt, typ = int(par["nt"]), par["dt"], par["typ"]
    nh, nv = h.size, v.size
    dout = cohc_fb(din, v, h, typ, nt, nv, nh, dt, operator, verb)
    ncol = nh if operator == 1 else nv
    if isinstance(dout, torch.Tensor):
        return dout.view(ncol, nt).t()
    return dout.reshape(nt, ncol, order="F")


def cohc_batch(windows, par, operator=-1, verb=0):
    """cohc (das.py:92) of many windows of the same shape in one launch (the
    DAS detection loop over the windows of a record): `windows` is a list of
    (nt, nh) arrays for operator -1 ((nt, nv) for 1) or one (nwin, nt, n)
    array; returns the list of results, each what cohc gives for that
    window.  The parabolic hmax state is updated once, as one cohc call."""
    h, v = _host_f32(par["h"], "h"), _host_f32(par["v"], "v")
    nt, dt, typ = int(par["nt"]), par["dt"], int(par["typ"])
    nh, nv = h.size, v.size
    if operator not in (1, -1):
        raise ValueError(f"cohc_batch: operator must be 1 or -1, got {operator}")
    wins = list(windows)
    if not wins:
        return []
    ncol_in = nv if operator == 1 else nh
    for w in wins:
        if tuple(w.shape) != (nt, ncol_in):
            raise ValueError(f"cohc_batch: window of shape {tuple(w.shape)}, expected "
                             f"{(nt, ncol_in)}")
    if typ not in (1, 2, 3):
        typ = 1
    if typ == 2:
        coh_state.update(h)
    if not _coh_indices_usable(v, h, typ, nt, dt, coh_state.hmax):
        raise ValueError("cohc_batch: curve sample indices not finite or beyond 2e9 samples")
    parts = [_to_dev_flat(w) for w in wins]
    x = torch.cat([t for t, _ in parts])
    dev = x.device
    out = D.coherence_batch(x, torch.from_numpy(v).to(dev), torch.from_numpy(h).to(dev), typ, nt,
                            len(wins), dt, operator, coh_state.hmax)
    ncol = nh if operator == 1 else nv
    res = out.view(len(wins), ncol, nt).transpose(1, 2)
    if parts[0][1]:
        return [r for r in res]
    host = res.cpu().numpy()
    return [np.ascontiguousarray(r) for r in host]


# --------------------------------------------------------------------------
# plane-wave painting (rgt.py / paint_cfuns.c cpaint2d)
# --------------------------------------------------------------------------
def cpaint2d(dip, trace, n1, n2, order, i0, eps, verb):
    """cpaint2d "OOiiiifi" (paint_cfuns.c:1861): the flat column-major slopes
    dip (n1 n2 values) and the seed trace (n1 values) painted from trace i0;
    returns the flat float32 section (a CUDA tensor for a tensor in).  Prints
    the reference's parameter line (it prints it whatever verb is).  Raises
    ValueError where the reference prints "Dimension mismatch" and returns
    NULL, for a seed of fewer than n1 values and for i0 outside [0, n2)
    (the reference reads and writes out of bounds there)."""
    n1, n2, order, i0 = int(n1), int(n2), int(order), int(i0)
    print("n1=%d,n2=%d,order=%d,i0=%d,eps=%g,verb=%d"
          % (n1, n2, order, i0, float(np.float32(eps)), int(verb)))
    p, as_t = _to_dev_flat(dip)
    if p.numel() != n1 * n2:
        raise ValueError(f"Dimension mismatch, N_input = {p.numel()}, N_data = {n1 * n2}")
    t, _ = _to_dev_flat(trace)
    if t.numel() < n1:
        raise ValueError(f"cpaint2d: the seed trace has {t.numel()} values, expected {n1}")
    if not 0 <= i0 < n2:
        raise ValueError(f"cpaint2d: reference trace i0 = {i0} outside [0, {n2})")
    if n1 < 4:
        raise ValueError("cpaint2d: n1 must be at least 4")
    out = D.paint2d(p, t[:n1].contiguous(), n1, n2, order, i0, eps)
    return out if as_t else out.cpu().numpy()


def pwpaintc(dip, trace, order=1, i0=0, eps=0.01, verb=False):
    """pwpaintc (rgt.py:51): plane-wave painting of the seed trace along the
    (n1, n2) slopes dip from trace i0; returns the (n1, n2) painted section
    (a CUDA tensor for a tensor in)."""
    n1, n2 = (int(x) for x in dip.shape)
    dout = cpaint2d(dip, trace, n1, n2, order, i0, eps, verb)
    if isinstance(dout, torch.Tensor):
        return _from_dev_flat(dout, (n1, n2), True)
    return dout.reshape(n1, n2, order="F")


def pwpaintc_batch(dips, traces, order=1, i0=0, eps=0.01):
    """pwpaintc (rgt.py:51) of many (n1, n2) sections of one size in one
    launch: `dips` a list of slope sections, `traces` their seed traces;
    returns the list of painted sections, each what pwpaintc gives."""
    dips, traces = list(dips), list(traces)
    if not dips or len(dips) != len(traces):
        raise ValueError("pwpaintc_batch: as many seed traces as sections, at least one")
    n1, n2 = (int(x) for x in dips[0].shape)
    if any(tuple(p.shape) != (n1, n2) for p in dips):
        raise ValueError("pwpaintc_batch: the sections must have one size")
    if not 0 <= int(i0) < n2 or n1 < 4:
        raise ValueError("pwpaintc_batch: i0 outside [0, n2) or n1 < 4")
    pp = [_to_dev_flat(p) for p in dips]
    tt = [_to_dev_flat(t)[0] for t in traces]
    if any(t.numel() < n1 for t in tt):
        raise ValueError(f"pwpaintc_batch: seed traces need {n1} values")
    p = torch.cat([x for x, _ in pp])
    t = torch.cat([x[:n1] for x in tt])
    out = D.paint2d_batch(p, t, n1, n2, len(dips), order, i0, eps).view(len(dips), n2, n1)
    res = out.transpose(1, 2)
    if pp[0][1]:
        return [r for r in res]
    return [np.ascontiguousarray(r) for r in res.cpu().numpy()]


def rgt(dip, o1=0, d1=0.004, order=1, i0=0, eps=0.01, verb=False):
    """rgt (rgt.py:4): relative geological time, the time axis o1 + d1 i1
    painted along the slopes dip from trace i0."""
    n1 = int(dip.shape[0])
    trace = np.linspace(0, d1 * (n1 - 1), n1) + o1
    if isinstance(dip, torch.Tensor):
        trace = torch.from_numpy(trace.astype(np.float32)).to(dip.device)
    return pwpaintc(dip, trace, order=order, i0=i0, eps=eps, verb=verb)


# --------------------------------------------------------------------------
# sparse-data interpolation (sint.py / soint2d_cfuns.c csint2d)
# --------------------------------------------------------------------------
def csint2d(din, dip, mask, n1, n2, niter, ns, order, verb, eps):
    """csint2d "OOOiiiiiif" (soint2d_cfuns.c:2421): the flat column-major
    section din (n1 n2 values, known where mask != 0) interpolated along the
    slopes dip by niter shaping CG iterations with the plane-wave smoothing
    of radius ns and accuracy order `order`; returns the flat float32 result
    (a CUDA tensor for a tensor in).  Prints the reference's parameter line
    (it prints it whatever verb is).  Raises ValueError where the reference
    prints "Dimension mismatch" and returns NULL, and for slopes or a mask
    of fewer than n1 n2 values (the reference reads past them)."""
    n1, n2, niter, ns, order = int(n1), int(n2), int(niter), int(ns), int(order)
    print("n1=%d,n2=%d,nw=%d,niter=%d,verb=%d,eps=%g"
          % (n1, n2, order, niter, int(verb), float(np.float32(eps))))
    n = n1 * n2
    d, as_t = _to_dev_flat(din)
    if d.numel() != n:
        raise ValueError(f"Dimension mismatch, N_input = {d.numel()}, N_data = {n}")
    p, _ = _to_dev_flat(dip)
    m, _ = _to_dev_flat(mask)
    if p.numel() < n or m.numel() < n:
        raise ValueError(f"csint2d: slopes and mask need {n} values each")
    if n1 < 4 or n2 < 1 or ns < 0 or order < 1 or niter < 0:
        raise ValueError("csint2d: invalid sizes or parameters")
    out = D.sint2d(d, p[:n].contiguous(), m[:n].contiguous(), n1, n2, niter, ns, order, eps)
    return out if as_t else out.cpu().numpy()


def sint2dc(din, mask, dip, niter=100, eps=0.01, ns=1, order=1, verb=1):
    """sint2dc (sint.py:61): interpolation of sparse data (e.g. well logs)
    in an (n1, n2) section along the slopes dip; known samples where mask !=
    0.  Returns the (n1, n2) section (a CUDA tensor for a tensor in)."""
    n1, n2 = (int(x) for x in din.shape)
    dout = csint2d(din, dip, mask, n1, n2, niter, ns, order, verb, eps)
    if isinstance(dout, torch.Tensor):
        return _from_dev_flat(dout, (n1, n2), True)
    return dout.reshape(n1, n2, order="F")


def csint3d(din, dipi, dipx, mask, n1, n2, n3, niter, ns1, ns2, order1, order2, verb, eps):
    """csint3d "OOOOiiiiiiiiif" (soint3d_cfuns.c:2510): the flat cube din
    (known where mask != 0) interpolated along the inline slopes dipi and
    the crossline slopes dipx; returns the flat float32 result (a CUDA
    tensor for a tensor in).  Prints the reference's parameter line (it
    prints it whatever verb is).  Raises ValueError where the reference
    prints "Dimension mismatch" and returns NULL, and for slopes or a mask
    of fewer values than the cube."""
    n1, n2, n3, niter = int(n1), int(n2), int(n3), int(niter)
    ns1, ns2, order1, order2 = int(ns1), int(ns2), int(order1), int(order2)
    print("n1=%d,n2=%d,n3=%d,ns1=%d,ns2=%d,nw1=%d,nw2=%d,niter=%d,verb=%d,eps=%g"
          % (n1, n2, n3, ns1, ns2, order1, order2, niter, int(verb), float(np.float32(eps))))
    n = n1 * n2 * n3
    d, as_t = _to_dev_flat(din)
    if d.numel() != n:
        raise ValueError(f"Dimension mismatch, N_input = {d.numel()}, N_data = {n}")
    pi, _ = _to_dev_flat(dipi)
    px, _ = _to_dev_flat(dipx)
    m, _ = _to_dev_flat(mask)
    if min(pi.numel(), px.numel(), m.numel()) < n:
        raise ValueError(f"csint3d: slopes and mask need {n} values each")
    if n1 < 4 or min(n2, n3) < 1 or min(ns1, ns2) < 0 or min(order1, order2) < 1 or niter < 0:
        raise ValueError("csint3d: invalid sizes or parameters")
    out = D.sint3d(d, pi[:n].contiguous(), px[:n].contiguous(), m[:n].contiguous(),
                   (n1, n2, n3), niter, (ns1, ns2), (order1, order2), eps)
    return out if as_t else out.cpu().numpy()


def sint3dc(din, mask, dipi, dipx, niter=100, eps=0.01, ns1=1, ns2=1, order1=1, order2=1,
            verb=1):
    """sint3dc (sint.py:97): interpolation of sparse data in an (n1, n2,
    n3) cube along the inline and crossline slopes; known samples where mask
    != 0.  Returns the cube (a CUDA tensor for a tensor in)."""
    n1, n2, n3 = (int(x) for x in din.shape)
    dout = csint3d(din, dipi, dipx, mask, n1, n2, n3, niter, ns1, ns2, order1, order2, verb, eps)
    if isinstance(dout, torch.Tensor):
        return _from_dev_flat(dout, (n1, n2, n3), True)
    return dout.reshape(n1, n2, n3, order="F")


# --------------------------------------------------------------------------
# FK dip filter (fk.py)
# --------------------------------------------------------------------------
def fkdip(d, w):
    """fkdip (fk.py:2): the part of the 2-D section d inside the FK cone of
    half-width w nk wavenumbers around k = 0 (nk = nextpow2 of the trace
    count), back in time and space, as float64 (the reference's numpy
    result type); the DAS chain subtracts it from the data.  float32 input
    keeps its forward FFTs in complex64 and float64 input in complex128, as
    numpy does (other types go through float64).  A CUDA tensor in gives a
    float64 CUDA tensor out.  w = 0
    raises ZeroDivisionError, as the reference's cone slope nrow / (w nk)
    does."""
    if len(d.shape) != 2:
        raise ValueError("fkdip: d must be 2-D")
    n1, n2 = (int(x) for x in d.shape)
    if float(w) == 0.0:
        raise ZeroDivisionError("float division by zero")
    if isinstance(d, torch.Tensor):
        t = d.to(device=_dev())
        if t.dtype not in (torch.float32, torch.float16, torch.bfloat16):
            t = t.to(torch.float64)
        elif t.dtype != torch.float32:
            t = t.to(torch.float32)
        t = t.t().contiguous().view(-1)
        out = D.fkdip(t, n1, n2, w)
        return out.view(n2, n1).t()
    a = np.asarray(d)
    dt = np.float32 if a.dtype in (np.float32, np.float16) else np.float64
    flat = np.ascontiguousarray(a.astype(dt, copy=False).reshape(-1, order="F"))
    t = torch.from_numpy(flat).to(_dev())
    out = D.fkdip(t, n1, n2, w)
    return out.cpu().numpy().reshape(n1, n2, order="F")
