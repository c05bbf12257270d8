"""Median selection (pwd_median.cuh): per-thread odd-even merge networks for
windows of up to 32 values, warp-cooperative rank selection beyond.  Both
return the reference's exact order statistic (sf_quantile,
pyseistr/src/sof_cfuns.c:1137-1163): bit for bit against the oracle, with
-0.0 == +0.0.  Windows longer than 96 values run too (the reference's mf
takes any length)."""
import numpy as np
import pytest

from gpu_util import need_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def O():
    from oracle import oracle

    return oracle


@pytest.fixture(scope="module")
def ps():
    need_gpu()
    import pyseistr_gb300

    return pyseistr_gb300


def _panel_case(O, ns, seed):
    rng = np.random.default_rng(seed)
    d = rng.standard_normal((48, 3 * ns + 5)).astype(np.float32)
    d[:, 2] = 0.0
    d[5:9, 4] = -0.0
    p = rng.uniform(-1.5, 1.5, d.shape).astype(np.float32)
    u = O.pwspray2d(d, p, ns, 2, 0.01)
    u[1, :, 3] = 0.75  # a column of ties
    return u


@pytest.mark.parametrize("ns,nmf,option", [(4, 9, 1), (7, 15, 1), (8, 17, 1), (15, 31, 1),
                                           (16, 33, 1), (20, 41, 1), (20, 41, 2), (40, 81, 1),
                                           (50, 101, 1), (50, 97, 2), (12, 25, 2)])
def test_panel_median_networks_and_warp_form(O, ps, ns, nmf, option):
    import torch
    from pyseistr_gb300 import device as D

    u = _panel_case(O, ns, ns * 7 + option)
    want = O.spray_median(u, nmf, option)
    got = D.panel_median(torch.from_numpy(np.ascontiguousarray(u)).cuda(), nmf,
                         option).cpu().numpy()
    assert np.array_equal(got, want), (ns, nmf, option)


@pytest.mark.parametrize("ns", [3, 16, 24, 50])
def test_somf2d_long_windows_vs_oracle(O, ps, ns):
    rng = np.random.default_rng(ns)
    d = rng.standard_normal((70, 2 * ns + 9)).astype(np.float32)
    p = rng.uniform(-1, 1, d.shape).astype(np.float32)
    got = ps.somf2dc(d, p, ns, 2, 0.01)
    want = O.somf2d(d, p, ns, 2, 0.01)
    assert np.array_equal(got, want)


def test_somf3d_window_99_vs_oracle(O, ps):
    """r1 = r2 = 7: somf3dc's window 2 r1 r2 + 1 = 99 (above the old cap)."""
    rng = np.random.default_rng(99)
    d = rng.standard_normal((40, 12, 11)).astype(np.float32)
    pi = rng.uniform(-1, 1, d.shape).astype(np.float32)
    px = rng.uniform(-1, 1, d.shape).astype(np.float32)
    got = ps.somf3dc(d, pi, px, 7, 7, 0.01, 2)
    want = O.somf3d(d, pi, px, 7, 7, 2)
    assert np.array_equal(got, want)
