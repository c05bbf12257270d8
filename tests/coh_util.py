"""Shared checks of the coherence tests.

The oracle marks NaN the model samples whose curve reaches past the end of
the data, where the reference reads an undefined value.  The library reads
that sample as 0; `zero_read_sample` evaluates such a model sample on its
own (float32 scalar arithmetic in the reference's order), so that those
samples are checked exactly too."""
import numpy as np

f32 = np.float32


def _index(itau, hh, vv, typ, dt, hmax):
    with np.errstate(all="ignore"):
        if typ == 2:
            t = f32(itau) * dt + hh * hh * vv / hmax / hmax
        elif typ == 3:
            tau = f32(itau) * dt
            hv = hh / vv
            t = np.sqrt(tau * tau + hv * hv)
        else:
            t = f32(itau) * dt + hh * vv
        return int(np.floor(t / dt) + f32(1))


def zero_read_sample(d, v, h, typ, nt, dt, hmax, itau, iv):
    """Coherence of model sample (itau, iv) of the flat data d with the
    sample past the end of d read as 0."""
    typ = typ if typ in (1, 2, 3) else 1
    dt, hmax = f32(dt), f32(hmax)
    nh = h.size
    num, den = f32(0), f32(0)
    for ih in range(nh):
        it = _index(itau, h[ih], v[iv], typ, dt, hmax)
        if 0 <= it <= nt:
            i = ih * nt + it
            y = d[i] if i < d.size else f32(0)
            num = f32(num + y)
            den = f32(den + f32(y * y))
    nn, nd = f32(num * num), f32(f32(nh) * den)
    return f32(np.float64(nn) / (np.float64(nd) + 1e-16))


def agrees(got, want, d, v, h, typ, nt, dt, hmax):
    """Bit for bit where the oracle is defined; where it is NaN (adjoint
    samples whose curve reaches past the end), the zero-read value."""
    got = np.asarray(got).reshape(-1, order="F")
    want = np.asarray(want).reshape(-1, order="F")
    undefined = np.isnan(want)
    if not np.array_equal(got[~undefined], want[~undefined]):
        return False
    if undefined.any():
        dflat = np.asarray(d, np.float32).reshape(-1, order="F")
        for k in np.flatnonzero(undefined):
            iv, itau = divmod(int(k), nt)
            if got[k] != zero_read_sample(dflat, v, h, typ, nt, dt, hmax, itau, iv):
                return False
    return True
