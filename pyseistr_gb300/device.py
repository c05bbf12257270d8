"""Device-resident entry points: flat, column-major float32 CUDA tensors in,
CUDA tensors out, enqueued on the current torch stream without host
synchronisation.

These are thin wrappers of the C ABI (include/pwd_gb300.h); each mirrors the
low-level reference entry it replaces (dipc, csomean2d, csomf2d, csomean3d,
csomf3d, csoint3d) with the sizes passed explicitly.  Workspaces come from
torch's caching allocator unless the caller passes one.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _as_flat(t, n, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != torch.float32:
        raise TypeError(f"{name} must be float32, got {t.dtype}")
    if t.numel() != n:
        raise ValueError(f"{name}: size {t.numel()} does not match the section size {n}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous (flat column-major)")
    return t.view(-1)


def _workspace(nbytes, device, ws=None):
    if nbytes == 0:
        raise ValueError("invalid sizes or parameters (workspace query returned 0)")
    if ws is not None:
        if ws.numel() * ws.element_size() < nbytes or ws.data_ptr() % 256:
            raise ValueError(f"workspace must be >= {nbytes} bytes and 256-byte aligned")
        return ws
    return torch.empty(nbytes, dtype=torch.uint8, device=device)


def dip(data, n1, n2, n3, niter=5, liter=20, order=2, rect=(10, 10, 1), mask=None, out=None,
        workspace=None):
    """Slopes of a section (n3 == 1, [n]) or cube (n3 > 1, [2n]: inline then crossline)."""
    L = _lib.load()
    n = n1 * n2 * n3
    data = _as_flat(data, n, "data")
    if mask is not None:
        mask = _as_flat(mask, n, "mask")
    rc = (ctypes.c_int * 3)(*[int(r) for r in rect])
    nbytes = L.pwd_dip_workspace_size(n1, n2, n3, order, rc, int(mask is not None))
    ws = _workspace(nbytes, data.device, workspace)
    nout = n if n3 == 1 else 2 * n
    if out is None:
        out = torch.empty(nout, dtype=torch.float32, device=data.device)
    _lib.check(L.pwd_dip(_ptr(data), _ptr(mask), _ptr(out), n1, n2, n3, niter, liter, order, rc,
                         _ptr(ws), ws.numel(), _stream()), "dip")
    return out


def somean2d(data, dip_, n1, n2, n3, ns, order, eps, adj=0, out=None, workspace=None):
    L = _lib.load()
    n = n1 * n2 * n3
    data, dip_ = _as_flat(data, n, "data"), _as_flat(dip_, n, "dip")
    ws = _workspace(L.pwd_somean2d_workspace_size(n1, n2, n3, ns, order), data.device, workspace)
    out = torch.empty_like(data) if out is None else out
    _lib.check(L.pwd_somean2d(_ptr(data), _ptr(dip_), _ptr(out), n1, n2, n3, ns, order, int(adj),
                              float(eps), _ptr(ws), ws.numel(), _stream()), "somean2d")
    return out


def somf2d(data, dip_, n1, n2, n3, ns, nmf, option, order, eps, out=None, workspace=None):
    L = _lib.load()
    n = n1 * n2 * n3
    data, dip_ = _as_flat(data, n, "data"), _as_flat(dip_, n, "dip")
    ws = _workspace(L.pwd_somf2d_workspace_size(n1, n2, n3, ns, nmf, option, order), data.device,
                    workspace)
    out = torch.empty_like(data) if out is None else out
    _lib.check(L.pwd_somf2d(_ptr(data), _ptr(dip_), _ptr(out), n1, n2, n3, ns, nmf, option, order,
                            float(eps), _ptr(ws), ws.numel(), _stream()), "somf2d")
    return out


def somean3d(data, dipi, dipx, n1, n2, n3, r1, r2, order, eps=0.01, out=None, workspace=None):
    L = _lib.load()
    n = n1 * n2 * n3
    data = _as_flat(data, n, "data")
    dipi, dipx = _as_flat(dipi, n, "dipi"), _as_flat(dipx, n, "dipx")
    ws = _workspace(L.pwd_somean3d_workspace_size(n1, n2, n3, r1, r2, order), data.device,
                    workspace)
    out = torch.empty_like(data) if out is None else out
    _lib.check(L.pwd_somean3d(_ptr(data), _ptr(dipi), _ptr(dipx), _ptr(out), n1, n2, n3, r1, r2,
                              order, float(eps), _ptr(ws), ws.numel(), _stream()), "somean3d")
    return out


def somf3d(data, dipi, dipx, n1, n2, n3, r1, r2, nmf, option, order, eps=0.01, out=None,
           workspace=None):
    L = _lib.load()
    n = n1 * n2 * n3
    data = _as_flat(data, n, "data")
    dipi, dipx = _as_flat(dipi, n, "dipi"), _as_flat(dipx, n, "dipx")
    ws = _workspace(L.pwd_somf3d_workspace_size(n1, n2, n3, r1, r2, nmf, option, order),
                    data.device, workspace)
    out = torch.empty_like(data) if out is None else out
    _lib.check(L.pwd_somf3d(_ptr(data), _ptr(dipi), _ptr(dipx), _ptr(out), n1, n2, n3, r1, r2, nmf,
                            option, order, float(eps), _ptr(ws), ws.numel(), _stream()), "somf3d")
    return out


def soint3d(data, mask, dipi, dipx, n1, n2, n3, order=1, nj1=1, nj2=1, niter=100, drift=0,
            seed=202223, hasmask=1, var=0.0, out=None, workspace=None):
    L = _lib.load()
    n = n1 * n2 * n3
    data = _as_flat(data, n, "data")
    mask = _as_flat(mask, n, "mask") if mask is not None else None
    dipi, dipx = _as_flat(dipi, n, "dipi"), _as_flat(dipx, n, "dipx")
    ws = _workspace(L.pwd_soint3d_workspace_size(n1, n2, n3, order), data.device, workspace)
    out = torch.empty_like(data) if out is None else out
    _lib.check(L.pwd_soint3d(_ptr(data), _ptr(mask), _ptr(dipi), _ptr(dipx), _ptr(out), n1, n2, n3,
                             order, nj1, nj2, niter, int(drift), int(seed), int(hasmask),
                             float(var), _ptr(ws), ws.numel(), _stream()), "soint3d")
    return out


def soint2d_prec(data, mask, dip1, dip2, n1, n2, order=1, niter=100, hasmask=1, twoplane=0,
                 out=None, workspace=None):
    """csoint2d with prec = 1: the interpolation preconditioned by the
    plane-wave integration along dip1 (and, when twoplane, chained with the
    one along dip2).  Synchronises the current stream."""
    L = _lib.load()
    n = n1 * n2
    data = _as_flat(data, n, "data")
    mask = _as_flat(mask, n, "mask") if mask is not None else None
    dip1 = _as_flat(dip1, n, "dip1")
    dip2 = _as_flat(dip2, n, "dip2") if twoplane else None
    ws = _workspace(L.pwd_soint2d_prec_workspace_size(n1, n2, order, int(bool(twoplane))),
                    data.device, workspace)
    out = torch.empty_like(data) if out is None else out
    _lib.check(L.pwd_soint2d_prec(_ptr(data), _ptr(mask), _ptr(dip1), _ptr(dip2), _ptr(out), n1,
                                  n2, order, niter, int(hasmask), int(bool(twoplane)), _ptr(ws),
                                  ws.numel(), _stream()), "soint2d_prec")
    return out


def panel_median(panels, nmf, option=1, out=None, workspace=None):
    """Median row (np-1)/2 of sprayed panels [ntr][np][n1] -> [ntr][n1]
    (the reference's mf/svmf as the somf filters use them)."""
    L = _lib.load()
    if not isinstance(panels, torch.Tensor) or not panels.is_cuda or panels.dim() != 3:
        raise TypeError("panels must be a 3-D CUDA tensor [ntr][np][n1]")
    if panels.dtype != torch.float32 or not panels.is_contiguous():
        raise TypeError("panels must be contiguous float32")
    ntr, npn, n1 = panels.shape
    ws = _workspace(L.pwd_panel_median_workspace_size(n1, npn, ntr, nmf, option), panels.device,
                    workspace)
    out = torch.empty((ntr, n1), dtype=torch.float32, device=panels.device) if out is None else out
    _lib.check(L.pwd_panel_median(_ptr(panels), _ptr(out), n1, npn, ntr, nmf, option, _ptr(ws),
                                  ws.numel(), _stream()), "panel_median")
    return out


def section_table(shapes, offsets=None, out_offsets=None):
    """ctypes array of pwd_section for sections of the given shapes packed
    one after another (or at the given element offsets)."""
    n = len(shapes)
    tab = (_lib.Section * n)()
    off = oof = 0
    for k, sh in enumerate(shapes):
        n1, n2 = int(sh[0]), int(sh[1])
        n3 = int(sh[2]) if len(sh) > 2 else 1
        tab[k].offset = off if offsets is None else int(offsets[k])
        tab[k].out_offset = oof if out_offsets is None else int(out_offsets[k])
        tab[k].n1, tab[k].n2, tab[k].n3 = n1, n2, n3
        size = n1 * n2 * n3
        off += size
        oof += size if n3 == 1 else 2 * size
    return tab, off, oof


def dip_batch(data, shapes, niter=5, liter=20, order=2, rect=(10, 10, 1), mask=None, out=None,
              workspace=None, mixed=False):
    """Slopes of many sections packed one after another in `data` (flat,
    each section column-major), all in one launch sequence.  Returns the
    packed slopes (n per 2-D section, 2n per cube).  mixed=True selects the
    mixed mode (FP32 taps, fused convolution smoothing, FP64 reductions)
    instead of the bit-faithful plain path."""
    L = _lib.load()
    tab, ntot, nout = section_table(shapes)
    data = _as_flat(data, ntot, "data")
    if mask is not None:
        mask = _as_flat(mask, ntot, "mask")
    rc = (ctypes.c_int * 3)(*[int(r) for r in rect])
    size_fn = L.pwd_dip_batch_mixed_workspace_size if mixed else L.pwd_dip_batch_workspace_size
    run_fn = L.pwd_dip_batch_mixed if mixed else L.pwd_dip_batch
    nbytes = size_fn(tab, len(shapes), order, rc, int(mask is not None))
    ws = _workspace(nbytes, data.device, workspace)
    if out is None:
        out = torch.empty(nout, dtype=torch.float32, device=data.device)
    _lib.check(run_fn(_ptr(data), _ptr(mask), _ptr(out), tab, len(shapes), niter, liter,
                      order, rc, _ptr(ws), ws.numel(), _stream()), "dip_batch")
    return out


class DipGraph:
    """Batched slope estimation captured once into a CUDA graph and replayed.

    The section table is uploaded once (pwd_dip_batch_prepare); the launch
    sequence of pwd_dip_batch_run (kernels and memsets only: the iteration
    control lives on the device) is captured on the current device and each
    call replays it on new contents of the fixed input buffer.  Results are
    those of dip_batch with the same arguments.
    """

    def __init__(self, shapes, niter=5, liter=20, order=2, rect=(10, 10, 1), mixed=False,
                 has_mask=False, device=None):
        L = _lib.load()
        dev = torch.device("cuda") if device is None else torch.device(device)
        self.tab, ntot, nout = section_table(shapes)
        self.nsec = len(shapes)
        self.args = (niter, liter, order)
        self.rect = (ctypes.c_int * 3)(*[int(r) for r in rect])
        self.mixed = int(bool(mixed))
        size_fn = L.pwd_dip_batch_mixed_workspace_size if mixed else L.pwd_dip_batch_workspace_size
        nbytes = size_fn(self.tab, self.nsec, order, self.rect, int(has_mask))
        self.ws = _workspace(nbytes, dev)
        self.data = torch.zeros(ntot, dtype=torch.float32, device=dev)
        self.mask = torch.ones(ntot, dtype=torch.float32, device=dev) if has_mask else None
        self.out = torch.empty(nout, dtype=torch.float32, device=dev)
        _lib.check(L.pwd_dip_batch_prepare(self.tab, self.nsec, order, self.rect, int(has_mask),
                                           self.mixed, _ptr(self.ws), self.ws.numel(), _stream()),
                   "dip_batch_prepare")
        self._run()  # once outside the capture (kernel attributes, lazy loading)
        torch.cuda.synchronize(dev)
        l0 = _lib.launch_count()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._run()
        self.launches = _lib.launch_count() - l0  # kernels in one replay
        torch.cuda.synchronize(dev)

    def _run(self):
        L = _lib.load()
        niter, liter, order = self.args
        _lib.check(L.pwd_dip_batch_run(_ptr(self.data), _ptr(self.mask), _ptr(self.out), self.tab,
                                       self.nsec, niter, liter, order, self.rect, self.mixed,
                                       _ptr(self.ws), self.ws.numel(), _stream()), "dip_batch_run")

    def __call__(self, data=None, mask=None):
        """Replays the estimation (on `data`/`mask` copied in first when
        given); returns the output buffer (reused by the next call)."""
        if data is not None:
            self.data.copy_(_as_flat(data, self.data.numel(), "data"))
        if mask is not None:
            if self.mask is None:
                raise ValueError("graph captured without a mask")
            self.mask.copy_(_as_flat(mask, self.mask.numel(), "mask"))
        self.graph.replay()
        return self.out


def soint3d_batch(data, mask, dips, shapes, order=1, niter=100, nj1=1, nj2=1, drift=0,
                  hasmask=1, out=None, workspace=None):
    """Interpolation of many cubes packed one after another in `data` and
    `mask`, with their slopes `dips` as dip_batch returns them."""
    L = _lib.load()
    tab, ntot, nout = section_table(shapes)
    data = _as_flat(data, ntot, "data")
    mask = _as_flat(mask, ntot, "mask") if mask is not None else None
    dips = _as_flat(dips, nout, "dips")
    ws = _workspace(L.pwd_soint3d_batch_workspace_size(tab, len(shapes), order), data.device,
                    workspace)
    out = torch.empty_like(data) if out is None else out
    _lib.check(L.pwd_soint3d_batch(_ptr(data), _ptr(mask), _ptr(dips), _ptr(out), tab, len(shapes),
                                   order, nj1, nj2, niter, int(drift), int(hasmask), _ptr(ws),
                                   ws.numel(), _stream()), "soint3d_batch")
    return out


def soint2d_prec_batch(data, mask, dip1, dip2, shapes, order=1, niter=100, hasmask=1,
                       twoplane=0, out=None, workspace=None):
    """csoint2d(prec=1) of many 2-D sections packed one after another in
    `data`, `mask` and `out`, their slopes `dip1` (and, when twoplane, the
    second planes' `dip2`) packed the same way, as dip_batch returns them:
    one CTA per section.  Synchronises the current stream."""
    L = _lib.load()
    tab, ntot, nout = section_table(shapes)
    data = _as_flat(data, ntot, "data")
    mask = _as_flat(mask, ntot, "mask") if mask is not None else None
    dip1 = _as_flat(dip1, nout, "dip1")
    dip2 = _as_flat(dip2, nout, "dip2") if twoplane else None
    tp = int(bool(twoplane))
    ws = _workspace(L.pwd_soint2d_prec_batch_workspace_size(tab, len(shapes), order, tp),
                    data.device, workspace)
    out = torch.empty_like(data) if out is None else out
    _lib.check(L.pwd_soint2d_prec_batch(_ptr(data), _ptr(mask), _ptr(dip1), _ptr(dip2), _ptr(out),
                                        tab, len(shapes), order, niter, int(hasmask), tp,
                                        _ptr(ws), ws.numel(), _stream()), "soint2d_prec_batch")
    return out


FILTER_MEAN, FILTER_MEAN_ADJ, FILTER_MEDIAN = 1, 2, 3


def sofilter2d_batch(data, dip_, shapes, ns, order=2, eps=0.01, filter=FILTER_MEAN, nmf=None,
                     option=1, out=None, workspace=None):
    """Structure-oriented mean (filter 1), adjoint mean (2) or median (3) of
    many 2-D sections packed one after another in `data` / `dip_`."""
    L = _lib.load()
    tab, ntot, _ = section_table(shapes, out_offsets=None)
    for k in range(len(shapes)):  # filter output uses the data layout
        tab[k].out_offset = tab[k].offset
    data, dip_ = _as_flat(data, ntot, "data"), _as_flat(dip_, ntot, "dip")
    nmf = 2 * ns + 1 if nmf is None else nmf
    nbytes = L.pwd_sofilter2d_batch_workspace_size(tab, len(shapes), ns, order, filter, nmf, option)
    ws = _workspace(nbytes, data.device, workspace)
    out = torch.empty_like(data) if out is None else out
    _lib.check(L.pwd_sofilter2d_batch(_ptr(data), _ptr(dip_), _ptr(out), tab, len(shapes), ns,
                                      order, filter, nmf, option, float(eps), _ptr(ws), ws.numel(),
                                      _stream()), "sofilter2d_batch")
    return out


def _patch_dims(n, l, s):
    n, l, s = (list(v) + [1] * (3 - len(v)) for v in (n, l, s))
    return n, l, s


def patch_count(n, l, s):
    """Number of windows of patch2d / patch3d (0 for invalid sizes)."""
    n, l, s = _patch_dims(n, l, s)
    return int(_lib.load().pwd_patch_count(*n, *l, *s))


def patch(a, n, l, s, out=None):
    """Windows of the column-major array `a` (flat CUDA float32, n = (n1, n2[,
    n3])) as a [npatch, prod(l)] tensor, each row a window flattened
    column-major (pwd_patch)."""
    L = _lib.load()
    nn, ll, ss = _patch_dims(n, l, s)
    npatch = int(L.pwd_patch_count(*nn, *ll, *ss))
    if npatch == 0:
        raise ValueError("invalid patch sizes")
    a = _as_flat(a, nn[0] * nn[1] * nn[2], "a")
    m = ll[0] * ll[1] * ll[2]
    if out is None:
        out = torch.empty((npatch, m), dtype=torch.float32, device=a.device)
    _lib.check(L.pwd_patch(_ptr(a), _ptr(out), *nn, *ll, *ss, _stream()), "patch")
    return out


def patch_inv(x, n, l, s, out=None):
    """Overlap-add of the windows x [npatch, prod(l)] back into a flat
    column-major array of shape n (pwd_patch_inv)."""
    L = _lib.load()
    nn, ll, ss = _patch_dims(n, l, s)
    npatch = int(L.pwd_patch_count(*nn, *ll, *ss))
    if npatch == 0:
        raise ValueError("invalid patch sizes")
    x = _as_flat(x, npatch * ll[0] * ll[1] * ll[2], "x")
    if out is None:
        out = torch.empty(nn[0] * nn[1] * nn[2], dtype=torch.float32, device=x.device)
    _lib.check(L.pwd_patch_inv(_ptr(x), _ptr(out), *nn, *ll, *ss, _stream()), "patch_inv")
    return out


def bandpass(d, n, dt, flo, fhi, nplo, nphi, phase, out=None):
    """Butterworth band-pass of every trace of the flat column-major CUDA
    float32 array `d` of shape n = (n1, n2, n3) (pwd_bandpass); `out` may be
    `d` itself."""
    L = _lib.load()
    n1, n2, n3 = (int(v) for v in n)
    d = _as_flat(d, n1 * n2 * n3, "d")
    if out is None:
        out = torch.empty_like(d)
    _lib.check(L.pwd_bandpass(_ptr(d), _ptr(out), n1, n2, n3, float(dt), float(flo),
                              float(fhi), int(nplo), int(nphi), int(phase), _stream()),
               "bandpass")
    return out


def coherence(x, v, h, typ, nt, dt, forw, hmax, out=None):
    """Radon coherence (pwd_coherence) of the flat column-major CUDA float32
    array `x`: forw = 1 maps the model [nv][nt] to the data [nh][nt], forw =
    -1 the data to the coherence model; v, h CUDA float32 vectors; hmax the
    parabolic normaliser kept by the caller."""
    L = _lib.load()
    nt, nv, nh = int(nt), int(v.numel()), int(h.numel())
    x = _as_flat(x, nt * (nv if forw == 1 else nh), "x")
    v = _as_flat(v, nv, "v")
    h = _as_flat(h, nh, "h")
    if out is None:
        out = torch.empty(nt * (nh if forw == 1 else nv), dtype=torch.float32, device=x.device)
    _lib.check(L.pwd_coherence(_ptr(x), _ptr(v), _ptr(h), int(typ), nt, nv, nh, float(dt),
                               int(forw), float(hmax), _ptr(out), _stream()), "coherence")
    return out


def coherence_batch(x, v, h, typ, nt, nwin, dt, forw, hmax, out=None):
    """pwd_coherence_batch: `nwin` windows stacked in the flat CUDA float32
    array x (each a model [nv][nt] for forw = 1, data [nh][nt] for -1)."""
    L = _lib.load()
    nt, nv, nh, nwin = int(nt), int(v.numel()), int(h.numel()), int(nwin)
    x = _as_flat(x, nwin * nt * (nv if forw == 1 else nh), "x")
    v = _as_flat(v, nv, "v")
    h = _as_flat(h, nh, "h")
    if out is None:
        out = torch.empty(nwin * nt * (nh if forw == 1 else nv), dtype=torch.float32,
                          device=x.device)
    _lib.check(L.pwd_coherence_batch(_ptr(x), _ptr(v), _ptr(h), int(typ), nt, nv, nh, nwin,
                                     float(dt), int(forw), float(hmax), _ptr(out), _stream()),
               "coherence_batch")
    return out


def paint2d(dip, seed, n1, n2, order, i0, eps, out=None, workspace=None):
    """Plane-wave painting (pwd_paint2d) of the seed trace (CUDA float32,
    n1 samples) from trace i0 along the flat column-major slopes `dip` of an
    (n1, n2) section; returns the flat painted section."""
    L = _lib.load()
    n1, n2, order, i0 = int(n1), int(n2), int(order), int(i0)
    dip = _as_flat(dip, n1 * n2, "dip")
    seed = _as_flat(seed, n1, "seed")
    ws = _workspace(L.pwd_paint2d_workspace_size(n1, order), dip.device, workspace)
    if out is None:
        out = torch.empty(n1 * n2, dtype=torch.float32, device=dip.device)
    _lib.check(L.pwd_paint2d(_ptr(dip), _ptr(seed), _ptr(out), n1, n2, order, i0, float(eps),
                             _ptr(ws), ws.numel() * ws.element_size(), _stream()), "paint2d")
    return out


def sint2d(din, dip, mask, n1, n2, niter, ns, order, eps, out=None, workspace=None):
    """Sparse-data interpolation (pwd_sint2d) of the flat column-major CUDA
    float32 section din (known where mask != 0) along the slopes dip;
    returns the flat interpolated section.  Synchronises the current stream
    during the call."""
    L = _lib.load()
    n1, n2 = int(n1), int(n2)
    n = n1 * n2
    din = _as_flat(din, n, "din")
    dip = _as_flat(dip, n, "dip")
    mask = _as_flat(mask, n, "mask")
    ws = _workspace(L.pwd_sint2d_workspace_size(n1, n2, int(ns), int(order)), din.device,
                    workspace)
    if out is None:
        out = torch.empty(n, dtype=torch.float32, device=din.device)
    _lib.check(L.pwd_sint2d(_ptr(din), _ptr(dip), _ptr(mask), _ptr(out), n1, n2, int(niter),
                            int(ns), int(order), float(eps), _ptr(ws),
                            ws.numel() * ws.element_size(), _stream()), "sint2d")
    return out


def sint3d(din, dipi, dipx, mask, n, niter, ns, order, eps, out=None, workspace=None):
    """Sparse-data interpolation of a cube (pwd_sint3d): n = (n1, n2, n3),
    ns = (ns1, ns2) and order = (order1, order2) for the inline and the
    crossline smoothing; flat column-major CUDA float32 arrays.  Synchronises
    the current stream during the call."""
    L = _lib.load()
    n1, n2, n3 = (int(v) for v in n)
    ns1, ns2 = (int(v) for v in ns)
    o1, o2 = (int(v) for v in order)
    m = n1 * n2 * n3
    din = _as_flat(din, m, "din")
    dipi = _as_flat(dipi, m, "dipi")
    dipx = _as_flat(dipx, m, "dipx")
    mask = _as_flat(mask, m, "mask")
    ws = _workspace(L.pwd_sint3d_workspace_size(n1, n2, n3, ns1, ns2, o1, o2), din.device,
                    workspace)
    if out is None:
        out = torch.empty(m, dtype=torch.float32, device=din.device)
    _lib.check(L.pwd_sint3d(_ptr(din), _ptr(dipi), _ptr(dipx), _ptr(mask), _ptr(out), n1, n2, n3,
                            int(niter), ns1, ns2, o1, o2, float(eps), _ptr(ws),
                            ws.numel() * ws.element_size(), _stream()), "sint3d")
    return out


def fkdip(d, n1, n2, w, out=None, workspace=None):
    """FK dip filter (pwd_fkdip / pwd_fkdip_f64) of the flat column-major
    CUDA section d (float32 or float64, whose precision the forward FFTs
    keep); returns the flat float64 cone-passed section."""
    L = _lib.load()
    n1, n2 = int(n1), int(n2)
    if not isinstance(d, torch.Tensor) or not d.is_cuda:
        raise TypeError("d must be a CUDA tensor")
    if d.dtype not in (torch.float32, torch.float64):
        raise TypeError(f"d must be float32 or float64, got {d.dtype}")
    if d.numel() != n1 * n2 or not d.is_contiguous():
        raise ValueError(f"d: size {d.numel()} does not match {n1} x {n2} or is not contiguous")
    f64 = d.dtype == torch.float64
    ws = _workspace(L.pwd_fkdip_workspace_size(n1, n2, int(f64)), d.device, workspace)
    if out is None:
        out = torch.empty(n1 * n2, dtype=torch.float64, device=d.device)
    fn = L.pwd_fkdip_f64 if f64 else L.pwd_fkdip
    _lib.check(fn(_ptr(d), _ptr(out), n1, n2, float(w), _ptr(ws), ws.numel() * ws.element_size(),
                  _stream()), "fkdip")
    return out


def paint2d_batch(dip, seed, n1, n2, nsec, order, i0, eps, out=None, workspace=None):
    """pwd_paint2d_batch: nsec (n1, n2) sections stacked in the flat CUDA
    float32 slopes `dip`, their seed traces stacked in `seed`."""
    L = _lib.load()
    n1, n2, nsec, order, i0 = int(n1), int(n2), int(nsec), int(order), int(i0)
    dip = _as_flat(dip, nsec * n1 * n2, "dip")
    seed = _as_flat(seed, nsec * n1, "seed")
    ws = _workspace(L.pwd_paint2d_batch_workspace_size(n1, nsec, order), dip.device, workspace)
    if out is None:
        out = torch.empty(nsec * n1 * n2, dtype=torch.float32, device=dip.device)
    _lib.check(L.pwd_paint2d_batch(_ptr(dip), _ptr(seed), _ptr(out), n1, n2, nsec, order, i0,
                                   float(eps), _ptr(ws), ws.numel() * ws.element_size(),
                                   _stream()), "paint2d_batch")
    return out
