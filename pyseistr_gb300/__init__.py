"""pyseistr_gb300: GB300-native plane-wave-destruction hot path of pyseistr.

Drop-in replacements of pyseistr's C-path entry points, computed by the
sm_103a kernels of libpwd_gb300.so:

    dip2dc, dip3dc                 local slopes (PWD + shaping division)
    somean2dc, somf2dc             2-D structure-oriented mean / median
    somean3dc, somf3dc             3-D structure-oriented mean / median
    soint3dc                       3-D structure-oriented interpolation
    soint2dc                       2-D structure-oriented interpolation
                                   (prec=1: preconditioned by plane-wave
                                   integration; soint2dc_batch for many
                                   sections at once)
    dipc, csomean2d, csomf2d,      the reference's low-level positional
    csomean3d, csomf3d, csoint3d,  entries
    csoint2d
    dip2dc_batch, somean2dc_batch, many sections of uneven size in one
    somf2dc_batch,                 launch sequence (same results as one
    dip_somean2d_batch,            call per section); the packed forms take
    dip_somean2d_packed,           flat (pinned) host tensors
    dip_soint3d_packed
    patch2d, patch3d,              windows of a section / cube and their
    patch2d_inv, patch3d_inv       overlap-add inverse (pyseistr/patch.py)
    bandpassc, cbp                 Butterworth band-pass along each trace
                                   (pyseistr/bp.py)
    cohc, cohc_fb, cohc_batch      time-domain Radon coherence along
                                   linear, parabolic or hyperbolic curves
                                   (pyseistr/das.py); many windows at once
    pwpaintc, rgt, cpaint2d,       plane-wave painting of a seed trace and
    pwpaintc_batch                 relative geological time (pyseistr/rgt.py)
    sint2dc, sint3dc,              sparse-data interpolation along the
    csint2d, csint3d               slopes (pyseistr/sint.py)
    fkdip                          FK dip (cone) filter (pyseistr/fk.py)

`pyseistr_gb300.device` has the device-resident (CUDA tensor) forms.
"""
from .api import (  # noqa: F401
    bandpassc,
    cbp,
    cohc,
    cohc_batch,
    cohc_fb,
    cpaint2d,
    csint2d,
    csint3d,
    csoint2d,
    csoint3d,
    csomean2d,
    csomean3d,
    csomf2d,
    csomf3d,
    dip2dc,
    dip2dc_batch,
    dip_somean2d_batch,
    dip_somean2d_packed,
    dip_soint3d_packed,
    dip3dc,
    dipc,
    fkdip,
    patch2d,
    patch2d_inv,
    patch3d,
    patch3d_inv,
    pwpaintc,
    pwpaintc_batch,
    rgt,
    sint2dc,
    sint3dc,
    soint2dc,
    soint2dc_batch,
    soint3dc,
    somean2dc,
    somean2dc_batch,
    somean3dc,
    somf2dc,
    somf2dc_batch,
    somf3dc,
)

__version__ = "0.1.0"
