"""Mixed-mode slope estimation (pwd_dip_batch_mixed) against the FP64
oracle: FP32 taps, the convolution form of the triangle smoothing fused with
the CG updates, FP64 reductions.  The bar is 1e-4 relative L2 against the
FP64 evaluation of the reference algorithm.  The plain FP32 path, which
reproduces the reference's float arithmetic, is 1e-5 to 7e-5 from FP64 on
the small inputs here, but up to 4e-3 on long sections of the batched
workload and 9e-2 on the full DAS record: the serial running sums of its
triangle smoothing lose precision along long lines."""
import numpy as np
import pytest

from gpu_util import need_gpu, rel_l2

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-4


@pytest.fixture(scope="module")
def D():
    need_gpu()
    from pyseistr_gb300 import device

    return device


@pytest.fixture(scope="module")
def O():
    from oracle import oracle

    return oracle


def _batch(D, secs, niter, liter, order, rect, mixed=True, mask=None):
    import torch

    shapes = [s.shape for s in secs]
    flat = np.concatenate([s.reshape(-1, order="F") for s in secs]).astype(np.float32)
    m = None
    if mask is not None:
        m = torch.from_numpy(np.concatenate([x.reshape(-1, order="F") for x in mask])
                             .astype(np.float32)).cuda()
    out = D.dip_batch(torch.from_numpy(flat).cuda(), shapes, niter, liter, order, rect,
                      mask=m, mixed=mixed).cpu().numpy()
    res, k = [], 0
    for s in secs:
        n = s.size
        if s.ndim == 3:
            res.append((out[k:k + n].reshape(s.shape, order="F"),
                        out[k + n:k + 2 * n].reshape(s.shape, order="F")))
            k += 2 * n
        else:
            res.append(out[k:k + n].reshape(s.shape, order="F"))
            k += n
    return res


def test_mixed_plain2d_vs_fp64(D, O):
    import workloads

    d = workloads.plain2d()
    got = _batch(D, [d], 5, 10, 2, (10, 10, 1))[0]
    want = O.dip2d(d, 5, 10, 2, (10, 10, 1), precision="f64")
    assert rel_l2(got, want) <= MIXED_TOL


def test_mixed_das_piece_vs_fp64(D, O):
    import workloads

    d = workloads.das2d(n1=600, n2=400, nev=8)
    got = _batch(D, [d], 5, 20, 2, (10, 10, 1))[0]
    want = O.dip2d(d, 5, 20, 2, (10, 10, 1), precision="f64")
    assert rel_l2(got, want) <= MIXED_TOL


def test_mixed_batch_sections_vs_fp64(D, O):
    """Uneven sections of the batched workload in one call, each against its
    own FP64 estimate."""
    import workloads

    secs = [s for s in workloads.batch2d(seed=5, count=8) if s.size <= 300_000][:5]
    got = _batch(D, secs, 5, 10, 2, (10, 10, 1))
    for s, g in zip(secs, got):
        want = O.dip2d(s, 5, 10, 2, (10, 10, 1), precision="f64")
        assert rel_l2(g, want) <= MIXED_TOL, s.shape


@pytest.mark.parametrize("order,rect", [(1, (3, 7, 1)), (3, (20, 2, 1)), (2, (1, 10, 1))])
def test_mixed_orders_and_radii_vs_fp64(D, O, order, rect):
    import workloads

    d = workloads.das2d(n1=300, n2=160, nev=5)
    got = _batch(D, [d], 4, 8, order, rect)[0]
    want = O.dip2d(d, 4, 8, order, rect, precision="f64")
    assert rel_l2(got, want) <= MIXED_TOL


def test_mixed_short_lines_vs_fp64(D, O):
    """Triangles longer than the lines (repeated mirroring)."""
    rng = np.random.default_rng(11)
    d = rng.standard_normal((40, 6)).astype(np.float32)
    got = _batch(D, [d], 3, 6, 2, (30, 12, 1))[0]
    want = O.dip2d(d, 3, 6, 2, (30, 12, 1), precision="f64")
    assert rel_l2(got, want) <= MIXED_TOL


def test_mixed_cube_vs_fp64(D, O):
    import workloads

    c = workloads.plain3d()[:, :30, :30].copy()
    gi, gx = _batch(D, [c], 5, 10, 2, (5, 5, 5))[0]
    wi, wx = O.dip3d(c, 5, 10, 2, (5, 5, 5), precision="f64")
    assert rel_l2(gi, wi) <= MIXED_TOL and rel_l2(gx, wx) <= MIXED_TOL


def test_mixed_mask_vs_fp64(D, O):
    import workloads

    d = workloads.das2d(n1=300, n2=120, nev=5)
    mask = np.ones_like(d)
    mask[:, 17] = 0.0
    mask[:, 60:63] = 0.0
    got = _batch(D, [d], 4, 8, 2, (8, 8, 1), mask=[mask])[0]
    want = O.dip2d(d, 4, 8, 2, (8, 8, 1), mask=mask, precision="f64")
    assert rel_l2(got, want) <= MIXED_TOL


def test_mixed_batch_equals_per_section_and_is_deterministic(D):
    """Tiles never straddle sections and the reductions run in a fixed
    order, so a batch gives each section's single-call result bit for bit,
    and reruns repeat it."""
    import workloads

    secs = [s[: max(64, s.shape[0] // 3), : max(20, s.shape[1] // 4)].copy()
            for s in workloads.batch2d(seed=9, count=5)]
    cube = workloads.plain3d()[:60, :11, :9].copy()
    allb = _batch(D, secs + [cube], 3, 6, 2, (6, 5, 3))
    again = _batch(D, secs + [cube], 3, 6, 2, (6, 5, 3))
    for k, s in enumerate(secs):
        one = _batch(D, [s], 3, 6, 2, (6, 5, 3))[0]
        assert np.array_equal(allb[k], one)
        assert np.array_equal(allb[k], again[k])
    one = _batch(D, [cube], 3, 6, 2, (6, 5, 3))[0]
    assert np.array_equal(allb[-1][0], one[0]) and np.array_equal(allb[-1][1], one[1])


def test_mixed_on_sections_where_fp32_drifts(D, O):
    """Sections of the batched workload on which the reference's own FP32
    arithmetic is furthest from FP64 (4.2e-3, 9.9e-4, 4.6e-4 relative L2).
    On the last two the mixed slopes are within the bar.  The first (2008 x
    67) is ill-conditioned for any float CG: the oracle with the smoothing
    evaluated in double and everything else in float (TRI_EXACT) is 7.3e-4
    from FP64 there; the mixed slopes must be at least three times closer
    than the reference's and within 1e-3."""
    import workloads

    allsecs = workloads.batch2d(count=64)
    secs = [allsecs[k] for k in (56, 18, 59)]
    got = _batch(D, secs, 5, 10, 2, (10, 10, 1))
    for k, (s, g) in enumerate(zip(secs, got)):
        want = O.dip2d(s, 5, 10, 2, (10, 10, 1), precision="f64")
        err = rel_l2(g, want)
        if k == 0:
            err32 = rel_l2(O.dip2d(s, 5, 10, 2, (10, 10, 1)), want)
            assert err <= 1e-3 and err <= err32 / 3, (s.shape, err, err32)
        else:
            assert err <= MIXED_TOL, (s.shape, err)


def _das_golden():
    import os

    path = os.path.join(os.path.dirname(__file__), "golden", "golden_das_full.npz")
    if not os.path.exists(path):
        pytest.skip("golden_das_full.npz not generated")
    return np.load(path)


def test_das_full_record_mixed_vs_fp64_and_plain_vs_reference(D):
    """The full 2000 x 5000 DAS record (dip2d niter 5, liter 20).  The
    reference's FP32 slopes are 8.8e-2 from FP64 over the record: the serial
    running sums of the triangle smoothing lose precision along the
    5000-trace lines, and the CG amplifies any rounding difference.  The
    plain path performs the reference's float operations but sums its FP64
    dot products (and the line search's residual energies) in another order.
    The fixture holds the oracle's FP32 restatement with exactly that
    summation order (flag GPU_DOTS) and everything else the reference's:
    the plain GPU slopes equal it bit for bit, so summation order is the
    whole difference from the reference's slopes (3.7e-2 over the record).
    The mixed slopes are within 1e-5 of FP64."""
    import workloads

    g = _das_golden()
    d = workloads.das2d(seed=2023)
    assert tuple(g["shape"]) == d.shape
    idx = g["idx"]
    mixed = _batch(D, [d], 5, 20, 2, (10, 10, 1), mixed=True)[0].reshape(-1, order="F")[idx]
    plain = _batch(D, [d], 5, 20, 2, (10, 10, 1), mixed=False)[0].reshape(-1, order="F")[idx]
    ref_err = float(g["ref32_rel_l2_vs_f64"])
    assert ref_err > 1e-2
    assert rel_l2(mixed, g["f64"]) <= 1e-5
    assert np.array_equal(plain, g["gpuorder32"])
    # the summation order's effect on the record, measured by the oracle
    gap = float(g["gpuorder32_rel_l2_vs_ref32"])
    assert rel_l2(plain, g["ref32"]) <= 1.1 * gap + 1e-3


@pytest.mark.parametrize("mixed", [False, True])
def test_dip_graph_replay_equals_direct_call(D, mixed):
    """The captured launch sequence replayed on new data gives the direct
    call's slopes bit for bit (plain and mixed), twice in a row."""
    import torch
    import workloads

    secs = [s[: max(64, s.shape[0] // 4), : max(20, s.shape[1] // 5)].copy()
            for s in workloads.batch2d(seed=21, count=4)]
    shapes = [s.shape for s in secs]
    flat = [np.concatenate([s.reshape(-1, order="F") for s in secs]).astype(np.float32)]
    flat.append((flat[0][::-1] * 0.5).copy())
    g = D.DipGraph(shapes, 3, 6, 2, (10, 10, 1), mixed=mixed)
    for f in flat:
        t = torch.from_numpy(f).cuda()
        want = D.dip_batch(t, shapes, 3, 6, 2, (10, 10, 1), mixed=mixed).cpu().numpy()
        got = g(t).cpu().numpy()
        assert np.array_equal(got, want)


def test_dipc_mixed_keyword_equals_batch(D, O):
    """dip2dc / dip3dc with mixed=True give the mixed batch's slopes for
    their one section (within the bar of FP64); the default stays the
    bit-faithful path."""
    import workloads
    import pyseistr_gb300 as ps

    d2 = workloads.plain2d()[:200, :60].copy()
    got = ps.dip2dc(d2, 3, 6, 2, rect=[10, 10, 1], mixed=True)
    assert np.array_equal(got, _batch(D, [d2], 3, 6, 2, (10, 10, 1))[0])
    plain = ps.dip2dc(d2, 3, 6, 2, rect=[10, 10, 1])
    assert np.array_equal(plain, _batch(D, [d2], 3, 6, 2, (10, 10, 1), mixed=False)[0])
    c = workloads.plain3d()[:60, :14, :11].copy()
    pi, px = ps.dip3dc(c, 2, 4, 2, rect=[5, 5, 5], mixed=True)
    wi, wx = _batch(D, [c], 2, 4, 2, (5, 5, 5))[0]
    assert np.array_equal(pi, wi) and np.array_equal(px, wx)
    fi, fx = O.dip3d(c, 2, 4, 2, (5, 5, 5), precision="f64")
    assert rel_l2(pi, fi) <= MIXED_TOL and rel_l2(px, fx) <= MIXED_TOL


def test_packed_host_api_equals_list_api(D):
    """dip_somean2d_packed on a pinned packed tensor returns the list API's
    slopes and filtered sections."""
    import torch
    import workloads
    import pyseistr_gb300 as ps

    secs = [s[: max(64, s.shape[0] // 4), : max(20, s.shape[1] // 5)].copy()
            for s in workloads.batch2d(seed=17, count=3)]
    shapes = [s.shape for s in secs]
    packed = torch.from_numpy(np.concatenate([s.reshape(-1, order="F") for s in secs])).pin_memory()
    for median in (False, True):
        p, f = ps.dip_somean2d_packed(packed, shapes, 3, 6, 2, [10, 10, 1], ns=4, median=median)
        pl, fl = ps.dip_somean2d_batch(secs, 3, 6, 2, [10, 10, 1], ns=4, median=median)
        k = 0
        for s, a, b in zip(secs, pl, fl):
            assert np.array_equal(p[k:k + s.size].numpy().reshape(s.shape, order="F"), a)
            assert np.array_equal(f[k:k + s.size].numpy().reshape(s.shape, order="F"), b)
            k += s.size


def test_batched_workload_every_section_vs_fp64(D):
    """The benchmark's batched workload at full size (512 sections of
    workloads.batch2d(seed=2023), dip2d(5, 10, rect 10,10,1) then
    somean2d(ns 6)) against the FP64 fixture made by
    tests/golden/make_golden_batch.py (at its 512 samples per section).  The
    mixed slopes and the mean filtered with them are within 1e-4 relative L2
    of the FP64 evaluation on every section but at most one; that one is an
    ill-conditioned section on which the reference's own FP32 is 2.5e-3 from
    FP64: it is held to 5e-4 and to a fifth of the reference's error (the
    float CG's rounding grows about tenfold per iteration there, so any
    float arithmetic lands 1e-5 .. 4e-4 from FP64: the oracle's float models
    measured there vary in that range with the rounding of single
    operations).  The plain path, the reference's float arithmetic, exceeds
    1e-4 on about sixty sections."""
    import os

    import torch
    import workloads

    path = os.path.join(os.path.dirname(__file__), "golden", "golden_batch_f64.npz")
    g = np.load(path)
    secs = workloads.batch2d(seed=2023, count=512)
    shapes = [s.shape for s in secs]
    assert [tuple(x) for x in g["shapes"]] == shapes
    flat = torch.from_numpy(np.concatenate([s.reshape(-1, order="F") for s in secs])).cuda()
    dip = D.dip_batch(flat, shapes, 5, 10, 2, (10, 10, 1), mixed=True)
    mean = D.sofilter2d_batch(flat, dip, shapes, 6, 2, 0.01)
    dip, mean = dip.cpu().numpy(), mean.cpu().numpy()
    cnt, idx, ref32 = g["count"], g["idx"], g["ref32_rel_l2_vs_f64"]
    k = j = 0
    over = []
    for q, (s, c) in enumerate(zip(secs, cnt)):
        ii = idx[j:j + c]
        es = rel_l2(dip[k:k + s.size][ii], g["dip64"][j:j + c])
        em = rel_l2(mean[k:k + s.size][ii], g["mean64"][j:j + c])
        if max(es, em) > MIXED_TOL:
            over.append((q, es, em, float(ref32[q])))
        k += s.size
        j += c
    assert len(over) <= 1, over
    for q, es, em, r in over:
        assert max(es, em) <= 5e-4 and es <= r / 5, (q, es, em, r)


def test_patches3d_masked_traces_vs_fp64(D):
    """The batched 3-D interpolation workload at full size (64 patches of
    workloads.patches3d(seed=2023): mixed dip3d(5, 10, rect 5,5,5) on each
    patch, then soint3d(order 2, niter 20) of the patch with half its traces
    masked): the reconstruction on the masked traces against the FP64
    evaluation of the same chain (tests/golden/make_golden_patches.py, 2048
    samples of the masked traces per patch), within 1e-4 relative L2 on
    every patch."""
    import os

    import torch
    import workloads

    path = os.path.join(os.path.dirname(__file__), "golden", "golden_patches_f64.npz")
    if not os.path.exists(path):
        pytest.skip("golden_patches_f64.npz not generated")
    g = np.load(path)
    pairs = workloads.patches3d(seed=2023, count=64)
    shapes = [d.shape for d, _ in pairs]
    assert [tuple(x) for x in g["shapes"]] == shapes
    full = torch.from_numpy(np.concatenate([d.reshape(-1, order="F") for d, _ in pairs])).cuda()
    mask = torch.from_numpy(np.concatenate([m.reshape(-1, order="F") for _, m in pairs])).cuda()
    p = D.dip_batch(full, shapes, 5, 10, 2, (5, 5, 5), mixed=True)
    x = D.soint3d_batch(full * mask, mask, p, shapes, order=2, niter=20).cpu().numpy()
    k = j = 0
    errs = []
    for (d, _), c in zip(pairs, g["count"]):
        ii = g["idx"][j:j + c]
        errs.append(rel_l2(x[k:k + d.size][ii], g["interp64"][j:j + c]))
        k += d.size
        j += c
    assert max(errs) <= MIXED_TOL, (max(errs), int(np.argmax(errs)))
