"""GPU results against the CPU oracle at sizes the oracle runs in seconds,
determinism, and size-independent properties at full workload sizes."""
import numpy as np
import pytest

from gpu_util import DIP_TOL, need_gpu, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ps():
    need_gpu()
    import pyseistr_gb300

    return pyseistr_gb300


@pytest.fixture(scope="module")
def O():
    from oracle import oracle

    return oracle


def test_dip2d_das_piece(ps, O):
    import workloads

    d = workloads.das2d(n1=600, n2=400, nev=8)
    got = ps.dip2dc(d, niter=5, liter=20, order=2, rect=[10, 10, 1])
    want = O.dip2d(d, 5, 20, 2, (10, 10, 1))
    assert rel_l2(got, want) <= DIP_TOL


def test_dip3d_plain3d(ps, O):
    import workloads

    c = workloads.plain3d()[:, :30, :30].copy()
    gi, gx = ps.dip3dc(c, 5, 10, 2, rect=[5, 5, 5])
    wi, wx = O.dip3d(c, 5, 10, 2, (5, 5, 5))
    assert rel_l2(gi, wi) <= DIP_TOL and rel_l2(gx, wx) <= DIP_TOL


@pytest.mark.parametrize("ns,order", [(4, 2), (10, 2), (6, 1)])
def test_somean_somf_2d(ps, O, ns, order):
    import workloads

    d = workloads.das2d(n1=300, n2=200, nev=6)
    p = O.dip2d(d, 2, 5, 2, (5, 5, 1))
    assert np.array_equal(ps.somean2dc(d, p, ns, order, 0.01), O.somean2d(d, p, ns, order, 0.01))
    assert np.array_equal(ps.somf2dc(d, p, ns, order, 0.01), O.somf2d(d, p, ns, order, 0.01))


def test_somf3d_r4(ps, O):
    import workloads

    c = workloads.plain3d()[:80, :16, :14].copy()
    pi, px = O.dip3d(c, 2, 4, 2, (3, 3, 3))
    assert np.array_equal(ps.somean3dc(c, pi, px, 4, 4, 0.01, 2), O.somean3d(c, pi, px, 4, 4, 2))
    assert np.array_equal(ps.somf3dc(c, pi, px, 4, 4, 0.01, 2), O.somf3d(c, pi, px, 4, 4, 2))


@pytest.mark.parametrize("r1,r2", [(5, 5), (6, 2), (3, 0)])
def test_somean3d_somf3d_radii_lane_groups(ps, O, r1, r2):
    """The 3-D spray runs each distance level of a source's tree on a group
    of 4, 8 or 16 lanes, set by the largest level: radius (5, 5) has a
    level of 12 cells (16 lanes), (6, 2) 8 lanes, (3, 0) 4 lanes."""
    import workloads

    c = workloads.plain3d()[:40, :14, :13].copy()
    pi, px = O.dip3d(c, 2, 4, 2, (3, 3, 3))
    assert np.array_equal(ps.somean3dc(c, pi, px, r1, r2, 0.01, 2),
                          O.somean3d(c, pi, px, r1, r2, 2))
    assert np.array_equal(ps.somf3dc(c, pi, px, r1, r2, 0.01, 2),
                          O.somf3d(c, pi, px, r1, r2, 2))


def test_median_selection_bit_exact_on_reference_spray(O):
    """The GPU median of sprayed panels equals the reference's quickselect
    when both are given the same (oracle-sprayed) values, including exact
    ties and signed zeros."""
    need_gpu()
    import torch

    rng = np.random.default_rng(3)
    d = rng.standard_normal((64, 40)).astype(np.float32)
    d[:, 5] = 0.0
    d[10:20, 7] = -0.0
    p = rng.uniform(-2, 2, d.shape).astype(np.float32)
    u = O.pwspray2d(d, p, 6, 2, 0.01)        # [n2][13][n1]
    u[3, :, 4] = 1.5                          # ties
    from pyseistr_gb300 import device as D

    tu = torch.from_numpy(np.ascontiguousarray(u)).cuda()
    for nmf, option in ((13, 1), (9, 1), (21, 1), (13, 2), (7, 2)):
        want = O.spray_median(u, nmf, option)
        got = D.panel_median(tu, nmf, option).cpu().numpy()
        assert np.array_equal(got, want), (nmf, option)


def test_determinism(ps):
    import workloads

    d = workloads.plain2d()
    a = ps.dip2dc(d, 5, 10, 2, rect=[10, 10, 1])
    b = ps.dip2dc(d, 5, 10, 2, rect=[10, 10, 1])
    assert np.array_equal(a, b)


def test_device_tensors_stay_on_device(ps, O):
    import torch
    import workloads

    d = workloads.plain2d()
    t = torch.from_numpy(d).cuda()
    p = ps.dip2dc(t, 5, 10, 2, rect=[10, 10, 1])
    assert isinstance(p, torch.Tensor) and p.is_cuda and tuple(p.shape) == d.shape
    q = ps.dip2dc(d, 5, 10, 2, rect=[10, 10, 1])
    assert np.array_equal(p.cpu().numpy(), q)


def test_bad_sizes_raise(ps):
    with pytest.raises(ValueError):
        ps.dipc(np.zeros(10, np.float32), 5, 3, 1, 1, 1, 2, 0.01, 1, 1e-6, 2, 2, 1, 0, 0)
    with pytest.raises(ValueError):
        ps.somf2dc(np.zeros((3, 5), np.float32), np.zeros((3, 5), np.float32), 2, 2, 0.01)


def test_full_size_properties(ps):
    """Configuration-3 size (2000 x 5000): the normalised mean of a constant
    field is that constant, and the median of a constant field is exact."""
    n1, n2 = 2000, 5000
    rng = np.random.default_rng(11)
    p = rng.uniform(-3, 3, (n1, n2)).astype(np.float32)
    ones = np.ones((n1, n2), np.float32)
    m = ps.somean2dc(ones, p, 10, 2, 0.01)
    assert np.all(np.isfinite(m))
    c = np.full((n1, n2), 0.75, np.float32)
    zp = np.zeros_like(p)
    med = ps.somf2dc(c, zp, 10, 2, 0.01)
    assert np.abs(med - 0.75).max() < 1e-3


def test_dip_batch_equals_per_section(ps):
    """A batch of uneven sections (2-D and 3-D mixed) gives bit for bit the
    slopes of one call per section."""
    import torch
    import workloads
    from pyseistr_gb300 import device as D

    secs = [s[: max(40, s.shape[0] // 4), : max(12, s.shape[1] // 6)].copy()
            for s in workloads.batch2d(count=6)]
    cube = workloads.plain3d()[:50, :9, :7].copy()
    shapes = [s.shape for s in secs] + [cube.shape]
    flat = np.concatenate([s.reshape(-1, order="F") for s in secs] + [cube.reshape(-1, order="F")])
    out = D.dip_batch(torch.from_numpy(flat).cuda(), shapes, 3, 6, 2, (5, 4, 3)).cpu().numpy()
    k = 0
    for s in secs:
        want = ps.dip2dc(s, 3, 6, 2, rect=[5, 4, 3])
        assert np.array_equal(out[k:k + s.size].reshape(s.shape, order="F"), want)
        k += s.size
    wi, wx = ps.dip3dc(cube, 3, 6, 2, rect=[5, 4, 3])
    assert np.array_equal(out[k:k + cube.size].reshape(cube.shape, order="F"), wi)
    assert np.array_equal(out[k + cube.size:].reshape(cube.shape, order="F"), wx)


@pytest.mark.parametrize("flt", [1, 2, 3])
def test_sofilter2d_batch_equals_per_section(ps, O, flt):
    import torch
    import workloads
    from pyseistr_gb300 import device as D

    secs = [s[: max(30, s.shape[0] // 5), : max(10, s.shape[1] // 8)].copy()
            for s in workloads.batch2d(count=5, seed=7)]
    dips = [O.dip2d(s, 2, 4, 2, (4, 4, 1)) for s in secs]
    shapes = [s.shape for s in secs]
    fl = lambda xs: np.concatenate([x.reshape(-1, order="F") for x in xs])
    out = D.sofilter2d_batch(torch.from_numpy(fl(secs)).cuda(), torch.from_numpy(fl(dips)).cuda(),
                             shapes, 3, 2, 0.01, filter=flt).cpu().numpy()
    k = 0
    for s, p in zip(secs, dips):
        if flt == 3:
            want = O.somf2d(s, p, 3, 2, 0.01)
        else:
            want = O.somean2d(s, p, 3, 2, 0.01, adj=flt - 1)
        assert np.array_equal(out[k:k + s.size].reshape(s.shape, order="F"), want)
        k += s.size
