#!/usr/bin/env python3
"""Benchmark of the PWD structural hot path on GB300.

One step = one pass of the hot path (slope estimation + structure-oriented
filter) over one batch of seeded synthetic input of a named workload:

  batch2d    512 sections, n1 ~ logU[256,2048] x n2 ~ logU[64,1024];
             dip2d (niter 5, liter 10, order 2, rect 10,10,1) + somean2d
             (ns 6, order 2, eps 0.01)                         [default]
  das2d      2000 x 5000 DAS-like record; dip2d (niter 5, liter 20) + somf2d
             (ns 10)
  plain2d    501 x 100; dip2d (5, 10) + somean2d + somf2d (ns 8)
  plain3d    201 x 60 x 60; dip3d (5, 10, rect 5,5,5) + somean3d + somf3d
             (r1 = r2 = 4)
  patches3d  64 cubes; dip3d + soint3d (order 2, niter 20)

Opt-in legs of the steps either side of the path: patch2d (patch2d +
patch2d_inv), bandpass2d (bandpassc of DAS records) and das_fkcoh (fkdip +
cohc of a DAS detection window).

metric: output samples per second (input samples fully processed by slope
estimation and filter per second).  `value` is timed on the device with
inputs resident in HBM; `e2e` is the same through the public drop-in API
(pyseistr_gb300.dip2dc / somean2dc ...) on host NumPy arrays, copies
included.  --impl reference times the reference algorithm on the host CPU
cores instead (the reference's own compiled C where importable, else the
bit-exact C restatement in oracle/), on a bounded sample of the workload.

Multi-GPU (torchrun): every rank runs its own replica of the workload
(weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import workloads as W  # noqa: E402

HBM_FALLBACK_GBS = 6800.0


# --------------------------------------------------------------------------
# workloads
# --------------------------------------------------------------------------
class Workload:
    name = ""

    def samples(self):
        raise NotImplementedError


class Batch2D(Workload):
    name = "batch2d"
    dip = dict(niter=5, liter=10, order=2, rect=(10, 10, 1))
    filt = dict(ns=6, order=2, eps=0.01)

    def __init__(self, seed, count=512):
        self.sections = W.batch2d(seed=seed, count=count)

    def samples(self):
        return int(sum(s.size for s in self.sections))

    def config(self):
        return {"workload": f"batch2d: {len(self.sections)} independent 2-D sections, "
                            "n1~logU[256,2048] x "
                            "n2~logU[64,1024]; dip2d(niter=5,liter=10,order=2,rect=10,10,1) + "
                            "somean2d(ns=6,order=2,eps=0.01)",
                "sections": len(self.sections), "samples_per_step": self.samples()}


class Das2D(Workload):
    name = "das2d"
    dip = dict(niter=5, liter=20, order=2, rect=(10, 10, 1))
    filt = dict(ns=10, order=2, eps=0.01)

    def __init__(self, seed):
        self.sections = [W.das2d(seed=seed)]

    def samples(self):
        return int(self.sections[0].size)

    def config(self):
        return {"workload": "das2d: 2000 x 5000 DAS-like record; dip2d(niter=5,liter=20,order=2,"
                            "rect=10,10,1) + somf2d(ns=10,order=2,eps=0.01)",
                "samples_per_step": self.samples()}


class Plain2D(Workload):
    name = "plain2d"
    dip = dict(niter=5, liter=10, order=2, rect=(10, 10, 1))
    filt = dict(ns=8, order=2, eps=0.01)

    def __init__(self, seed):
        self.sections = [W.plain2d(seed=seed)]

    def samples(self):
        return int(self.sections[0].size)

    def config(self):
        return {"workload": "plain2d: 501 x 100; dip2d(5,10,order 2,rect 10,10,1) + somean2d + "
                            "somf2d (ns 8, order 2, eps 0.01)", "samples_per_step": self.samples()}


class Plain3D(Workload):
    name = "plain3d"
    dip = dict(niter=5, liter=10, order=2, rect=(5, 5, 5))
    filt = dict(r1=4, r2=4, order=2, eps=0.01)

    def __init__(self, seed):
        self.sections = [W.plain3d(seed=seed)]

    def samples(self):
        return int(self.sections[0].size)

    def config(self):
        return {"workload": "plain3d: 201 x 60 x 60 cube; dip3d(5,10,order 2,rect 5,5,5) + "
                            "somean3d + somf3d (r1 = r2 = 4, order 2)",
                "samples_per_step": self.samples()}

    def cpu_sample(self, budget_s):
        c = self.sections[0]
        k = max(4, min(c.shape[2], int(budget_s * 0.02e6 / (c.shape[0] * c.shape[1]))))
        return [np.ascontiguousarray(c[:, :, :k])], f"sub-cube {c.shape[0]} x {c.shape[1]} x {k}"


class Patches3D(Workload):
    name = "patches3d"
    dip = dict(niter=5, liter=10, order=2, rect=(5, 5, 5))
    filt = dict(order=2, niter=20)

    def __init__(self, seed, count=64):
        pairs = W.patches3d(seed=seed, count=count)
        self.sections = [d for d, _ in pairs]
        self.masks = [m for _, m in pairs]

    def samples(self):
        return int(sum(s.size for s in self.sections))

    def config(self):
        return {"workload": f"patches3d: {len(self.sections)} cubes n1~U[128,512], "
                            "n2=n3~U[32,96], 50 % of traces masked; dip3d(5,10,order 2,"
                            "rect 5,5,5) on all cubes in one batch + soint3d(order 2, niter 20)",
                "sections": len(self.sections), "samples_per_step": self.samples()}

    def cpu_sample(self, budget_s):
        return [(self.sections[0], self.masks[0])], "the first patch"


WORKLOADS = {"batch2d": Batch2D, "das2d": Das2D, "plain2d": Plain2D, "plain3d": Plain3D,
             "patches3d": Patches3D}


def make_workload(args, rank=0):
    if args.workload == "batch2d":
        return Batch2D(seed=args.seed + rank, count=args.sections)
    if args.workload == "patches3d":
        return Patches3D(seed=args.seed + rank, count=min(args.sections, 64))
    return WORKLOADS[args.workload](seed=args.seed + rank)


# --------------------------------------------------------------------------
# GPU step (device-resident, batched) and the public-API (host) step
# --------------------------------------------------------------------------
class DeviceState:
    """Packed device copies of a workload's sections, outputs and workspaces."""

    def __init__(self, wl, dev):
        import torch
        from pyseistr_gb300 import device as D

        self.shapes = [s.shape for s in wl.sections]
        flat = np.concatenate([s.reshape(-1, order="F") for s in wl.sections])
        self.d = torch.from_numpy(flat).to(dev)
        _, _, nout = D.section_table(self.shapes)
        self.p = torch.empty(nout, dtype=torch.float32, device=dev)
        self.f = torch.empty_like(self.d)
        self.g = torch.empty_like(self.d) if wl.name in ("plain2d", "plain3d") else None
        if wl.name == "patches3d":  # interpolation inputs: masked data and the mask
            m = np.concatenate([x.reshape(-1, order="F") for x in wl.masks])
            self.m = torch.from_numpy(m).to(dev)
            self.dm = self.d * self.m
        self.D = D
        self.graph = None

    def capture(self, wl, mixed):
        """Captures the slope estimation into a CUDA graph on these inputs."""
        d = wl.dip
        self.graph = self.D.DipGraph(self.shapes, d["niter"], d["liter"], d["order"], d["rect"],
                                     mixed=mixed, device=self.d.device)
        self.graph.data.copy_(self.d)


def accuracy_vs_fp64(wl, st, seed):
    """Relative L2 distance of the step's outputs to the FP64 evaluation of
    the reference algorithm, from the committed fixtures (sampled indices):
    the batched workload's slopes and mean per section
    (tests/golden/golden_batch_f64.npz, 512 samples a section) and the DAS
    record's slopes (tests/golden/golden_das_full.npz, 32768 samples).
    None when no fixture matches the workload."""
    def rel(a, b):
        a, b = np.float64(a), np.float64(b)
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    g = os.path.join(ROOT, "tests", "golden")
    if wl.name == "batch2d" and seed == 2023 and len(st.shapes) == 512:
        path = os.path.join(g, "golden_batch_f64.npz")
        if not os.path.exists(path):
            return None
        z = np.load(path)
        if [tuple(x) for x in z["shapes"]] != [tuple(x) for x in st.shapes]:
            return None
        dip, mean = st.p.cpu().numpy(), st.f.cpu().numpy()
        k = j = 0
        es, em = [], []
        for shp, c in zip(st.shapes, z["count"]):
            n = int(np.prod(shp))
            ii = z["idx"][j:j + c]
            es.append(rel(dip[k:k + n][ii], z["dip64"][j:j + c]))
            em.append(rel(mean[k:k + n][ii], z["mean64"][j:j + c]))
            k += n
            j += c
        return {"slopes_rel_l2_max_section": max(es),
                "slopes_rel_l2_median_section": float(np.median(es)),
                "sections_over_1e-4": int(sum(max(a, b) > 1e-4 for a, b in zip(es, em))),
                "mean_rel_l2_max_section": max(em),
                "reference_fp32_slopes_rel_l2_max_section":
                float(np.max(z["ref32_rel_l2_vs_f64"])),
                "reference_fp32_sections_over_1e-4":
                int(np.sum(z["ref32_rel_l2_vs_f64"] > 1e-4)),
                "samples": "512 per section (tests/golden/golden_batch_f64.npz)"}
    if wl.name == "patches3d" and seed == 2023 and len(st.shapes) == 64:
        path = os.path.join(g, "golden_patches_f64.npz")
        if not os.path.exists(path):
            return None
        z = np.load(path)
        if [tuple(x) for x in z["shapes"]] != [tuple(x) for x in st.shapes]:
            return None
        x = st.f.cpu().numpy()
        k = j = 0
        es = []
        for shp, c in zip(st.shapes, z["count"]):
            n = int(np.prod(shp))
            es.append(rel(x[k:k + n][z["idx"][j:j + c]], z["interp64"][j:j + c]))
            k += n
            j += c
        return {"masked_traces_rel_l2_max_patch": max(es),
                "masked_traces_rel_l2_median_patch": float(np.median(es)),
                "reference_fp32_masked_traces_rel_l2_max_patch":
                float(np.max(z["ref32_rel_l2_vs_f64"])),
                "fp64_chain_vs_true_data_median_patch": float(np.median(z["f64_rel_l2_vs_truth"])),
                "samples": "2048 of the masked traces per patch "
                           "(tests/golden/golden_patches_f64.npz)"}
    if wl.name == "das2d" and seed == 2023:
        z = np.load(os.path.join(g, "golden_das_full.npz"))
        if tuple(z["shape"]) != tuple(st.shapes[0]):
            return None
        dip = st.p.cpu().numpy()
        return {"slopes_rel_l2": rel(dip[z["idx"]], z["f64"]),
                "reference_fp32_slopes_rel_l2": float(z["ref32_rel_l2_vs_f64"]),
                "samples": "32768 (tests/golden/golden_das_full.npz)"}
    return None


def gpu_step(wl, st, mixed=False):
    D = st.D
    d = wl.dip
    f = wl.filt
    if st.graph is not None and bool(st.graph.mixed) == mixed:
        st.graph()  # replay the captured slope estimation (inputs already in place)
        st.p.copy_(st.graph.out)
    else:
        D.dip_batch(st.d, st.shapes, d["niter"], d["liter"], d["order"], d["rect"], out=st.p,
                    mixed=mixed)
    if wl.name == "plain3d":
        n1, n2, n3 = st.shapes[0]
        n = n1 * n2 * n3
        pi, px = st.p[:n], st.p[n:]
        D.somean3d(st.d, pi, px, n1, n2, n3, f["r1"], f["r2"], f["order"], f["eps"], out=st.f)
        D.somf3d(st.d, pi, px, n1, n2, n3, f["r1"], f["r2"], 2 * f["r1"] * f["r2"] + 1, 1,
                 f["order"], f["eps"], out=st.g)
    elif wl.name == "patches3d":
        D.soint3d_batch(st.dm, st.m, st.p, st.shapes, order=f["order"], niter=f["niter"],
                        out=st.f)
    elif wl.name == "das2d":
        D.sofilter2d_batch(st.d, st.p, st.shapes, f["ns"], f["order"], f["eps"],
                           filter=D.FILTER_MEDIAN, out=st.f)
    else:
        D.sofilter2d_batch(st.d, st.p, st.shapes, f["ns"], f["order"], f["eps"],
                           filter=D.FILTER_MEAN, out=st.f)
        if wl.name == "plain2d":
            D.sofilter2d_batch(st.d, st.p, st.shapes, f["ns"], f["order"], f["eps"],
                               filter=D.FILTER_MEDIAN, out=st.g)


def api_step(wl, mixed=False, host=None):
    """The public batched API on host arrays: upload, slopes, filter,
    download.  Returns (h2d_bytes, d2h_bytes).  host = (packed pinned
    input, (pinned slope output, pinned filter output)) for the 2-D
    batched workloads."""
    import pyseistr_gb300 as ps

    d = wl.dip
    f = wl.filt
    nbytes = sum(s.nbytes for s in wl.sections)
    if host is not None and wl.name in ("batch2d", "das2d"):
        data, out = host
        ps.dip_somean2d_packed(data, [s.shape for s in wl.sections], niter=d["niter"],
                               liter=d["liter"], order=d["order"], rect=list(d["rect"]),
                               ns=f["ns"], eps=f["eps"], median=(wl.name == "das2d"),
                               mixed=mixed, out=out)
        return nbytes, 2 * nbytes
    if wl.name == "plain3d":
        c = wl.sections[0]
        pi, px = ps.dip3dc(c, d["niter"], d["liter"], d["order"], eps_dv=0.01, eps_cg=1,
                           tol_cg=1e-6, rect=list(d["rect"]), mixed=mixed)
        ps.somean3dc(c, pi, px, f["r1"], f["r2"], f["eps"], f["order"])
        ps.somf3dc(c, pi, px, f["r1"], f["r2"], f["eps"], f["order"])
        return 7 * nbytes, 4 * nbytes
    if wl.name == "patches3d":
        (data, mask), out = host
        ps.dip_soint3d_packed(data, mask, [s.shape for s in wl.sections], d["niter"],
                              d["liter"], d["order"], list(d["rect"]), f["order"], f["niter"],
                              mixed=mixed, out=out)
        return 2 * nbytes, nbytes
    p, out = ps.dip_somean2d_batch(wl.sections, niter=d["niter"], liter=d["liter"],
                                   order=d["order"], rect=list(d["rect"]), ns=f["ns"],
                                   eps=f["eps"], median=(wl.name == "das2d"), mixed=mixed)
    h2d, d2h = nbytes, 2 * nbytes
    if wl.name == "plain2d":
        ps.somf2dc_batch(wl.sections, p, f["ns"], f["order"], f["eps"])
        h2d += 2 * nbytes
        d2h += nbytes
    return h2d, d2h


# Algorithmic bytes per sample of each kernel family, averaged over the
# family's launches of one step (what the launches must read and write at
# minimum; every launch covers every section of the batch).
def fp32_peak_tflops():
    """FP32 FMA peak of this GPU, measured with the library's probe kernel
    (pwd_fp32_fma_probe: 8 independent FMA chains per thread, 8 blocks of
    256 threads per SM), best of 5 launches timed with CUDA events."""
    import ctypes

    import torch
    from pyseistr_gb300 import _lib

    lib = _lib.load()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads, iters = 8 * sms, 256, 16384
    out = torch.empty(blocks * threads, dtype=torch.float32, device="cuda")
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    best = None
    for _ in range(6):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        _lib.check(lib.pwd_fp32_fma_probe(ctypes.c_void_p(out.data_ptr()), blocks, threads,
                                          iters, st), "fp32 probe")
        b.record()
        b.synchronize()
        t = a.elapsed_time(b) / 1e3
        best = t if best is None else min(best, t)
    return 16.0 * iters * blocks * threads / best / 1e12


def spray_flops_per_sample(wl):
    """Algorithmic FP32 work of the spray and its filter per input sample
    (the pinned model: 2-D mean 148 ns + 220, 2-D median 74 ns + 220, 3-D
    (np - 1) x 47 + 880 per filter), for the workloads that spray."""
    f = wl.filt
    if wl.name == "batch2d":
        return 148 * f["ns"] + 220
    if wl.name == "das2d":
        return 74 * f["ns"] + 220
    if wl.name == "plain2d":
        return (148 * f["ns"] + 220) + (74 * f["ns"] + 220)
    if wl.name == "plain3d":
        npc = (2 * f["r1"] + 1) * (2 * f["r2"] + 1)
        return 2 * ((npc - 1) * 47 + 880)
    return 0


def family_bytes(wl, launches, mixed=False):
    """Average algorithmic bytes per launch of each family for one step."""
    n = wl.samples()
    d = wl.dip
    liter, niter = d["liter"], d["niter"]
    out = {}
    for fam, cnt in launches.items():
        if cnt == 0:
            continue
        if fam == "pwd":
            # residual: read u, p, write r (12 B); derivative + normalisation:
            # read u, p, r, write num, den, p0 (24 B); line-search trials:
            # read u, p0, dp, write p (16 B)
            trials = max(0, cnt - 1 - niter)
            bps = (12.0 + 24.0 * niter + 16.0 * trials) / max(1, 1 + niter + trials)
        elif fam == "cg" and mixed and d["rect"][2] > 1 and wl.name in ("plain3d", "patches3d"):
            # cubes, per CG iteration: axis 0 with the step and gradient 24
            # (read x, W, num, sx; write x, t; 20 first), axis 1 8, axis 2
            # with gp 20 (12 first), axes 0 and 1 of gp 8 in one pass (two
            # passes of 8 where the fused pass is not used), axis 2 with the
            # update 28 (read t, gp, W, sp, sx; write sp, sx; 20 first);
            # scale 28 and final step 12 per Gauss-Newton iteration
            r0, r1 = d["rect"][0], d["rect"][1]
            fused = (r0 == r1 and r0 in (5, 10) and os.environ.get("PWD_CONV01") != "0"
                     and os.environ.get("PWD_CONV1_PAIR") != "1")
            gp01, k = (8, 5) if fused else (16, 6)
            per_outer = 28 + (20 + 8 + 12 + gp01 + 20) + (liter - 1) * (80 + gp01) + 12
            bps = per_outer / (2.0 + k * liter)
        elif fam == "cg" and mixed:
            # per CG iteration: axis 0 with the step and gradient 24 (read
            # x, W, num, sx; write x, t; 20 first), axis 1 with gp 20 (12
            # first), axis 0 of gp 8, axis 1 with the conjugate update 28
            # (read t, gp, W, sp, sx; write sp, sx; 20 first); scale 28 and
            # final step 12 per Gauss-Newton iteration
            per_outer = 28 + (20 + 12 + 8 + 20) + (liter - 1) * 80 + 12
            bps = per_outer / (2.0 + 4.0 * liter)
        elif fam == "cg":
            # per Gauss-Newton iteration: scale 28, first gradient 16, later
            # step+gradient 44, gp 16, first update 24, later updates 36,
            # final step 12 (bytes per sample)
            per_outer = 28 + 16 + 44 * (liter - 1) + 16 * liter + 24 + 36 * (liter - 1) + 12
            bps = per_outer / (2.0 + 3.0 * liter)
        elif fam == "triangle":
            bps = 8.0  # each line sweep reads and writes its axis once
        elif fam == "spray":
            bps = 8.0  # read the data and the slopes
        else:
            bps = 12.0
        out[fam] = bps * n
    return out


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None

    def __enter__(self):
        self.first = []
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.idx)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            # the sampler is running before the timed region starts: its
            # first sample is taken just before, the others during the region
            ln = self.proc.stdout.readline()
            if ln.strip():
                self.first = [ln.strip()]
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = list(self.first)
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines += [ln for ln in out.splitlines() if ln.strip()]
        return False

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        loaded = [v for v in sm if v > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------
# CPU baseline (reference algorithm on host cores)
# --------------------------------------------------------------------------
def _ref_modules():
    """The reference's own compiled C extensions, when importable here."""
    path = os.path.join(ROOT, "oracle", "_ref")
    if not os.path.isdir(path):
        return None
    sys.path.insert(0, path)
    try:
        import dipcfun  # noqa: F401
        import sofcfun  # noqa: F401
        return "reference"
    except ImportError:
        return None
    finally:
        sys.path.remove(path)


def cpu_section(args):
    """Slope + filter of one section on the CPU; returns samples processed."""
    wl_name, sec, kind = args
    wl = WORKLOADS[wl_name]
    d = wl.dip
    f = wl.filt
    if wl_name in ("plain3d", "patches3d"):  # the port (float oracle)
        from oracle import oracle as O

        if wl_name == "plain3d":
            pi, px = O.dip3d(sec, d["niter"], d["liter"], d["order"], d["rect"])
            O.somean3d(sec, pi, px, f["r1"], f["r2"], f["order"])
            O.somf3d(sec, pi, px, f["r1"], f["r2"], f["order"])
            return sec.size
        c, m = sec
        pi, px = O.dip3d(c, d["niter"], d["liter"], d["order"], d["rect"])
        O.soint3d(c * m, m, pi, px, order=f["order"], niter=f["niter"])
        return c.size
    n1, n2 = sec.shape
    if kind == "reference":
        path = os.path.join(ROOT, "oracle", "_ref")
        if path not in sys.path:
            sys.path.insert(0, path)
        import dipcfun
        import sofcfun

        fd = os.dup(1)
        nul = os.open(os.devnull, os.O_WRONLY)
        os.dup2(nul, 1)
        try:
            flat = np.float32(sec.flatten(order="F"))
            p = dipcfun.dipc(flat, n1, n2, 1, d["niter"], d["liter"], d["order"], 0.01, 1.0, 1e-6,
                             d["rect"][0], d["rect"][1], d["rect"][2], 0, 0)
            if wl_name == "das2d":
                sofcfun.csomf2d(flat, p, n1, n2, 1, f["ns"], 2 * f["ns"] + 1, 1, f["order"],
                                f["eps"], 0)
            else:
                sofcfun.csomean2d(flat, p, n1, n2, 1, f["ns"], f["order"], 0, f["eps"], 0)
                if wl_name == "plain2d":
                    sofcfun.csomf2d(flat, p, n1, n2, 1, f["ns"], 2 * f["ns"] + 1, 1, f["order"],
                                    f["eps"], 0)
        finally:
            os.dup2(fd, 1)
            os.close(fd)
            os.close(nul)
    else:
        from oracle import oracle as O

        p = O.dip2d(sec, d["niter"], d["liter"], d["order"], d["rect"])
        if wl_name == "das2d":
            O.somf2d(sec, p, f["ns"], f["order"], f["eps"])
        else:
            O.somean2d(sec, p, f["ns"], f["order"], f["eps"])
            if wl_name == "plain2d":
                O.somf2d(sec, p, f["ns"], f["order"], f["eps"])
    return sec.size


def cpu_sample(wl, budget_s):
    """Sections of the workload whose CPU processing fits about budget_s."""
    if hasattr(wl, "cpu_sample"):
        return wl.cpu_sample(budget_s)
    secs = wl.sections
    if len(secs) == 1:
        return secs, "the whole workload"
    # the reference's speed is ~0.15 Msamples/s per core for dip + filter
    target = 0.15e6 * budget_s
    out, tot = [], 0
    for s in secs:
        out.append(s)
        tot += s.size
        if tot >= target:
            break
    return out, f"first {len(out)} of {len(secs)} sections ({tot} samples)"


def time_cpu(wl, sample, kind, workers):
    if workers <= 1:
        t0 = time.perf_counter()
        n = sum(cpu_section((wl.name, s, kind)) for s in sample)
        return n, time.perf_counter() - t0
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        pool.map(cpu_section, [(wl.name, s, kind) for s in sample[:workers]], chunksize=1)  # warm
        t0 = time.perf_counter()
        n = sum(pool.map(cpu_section, [(wl.name, s, kind) for s in sample], chunksize=1))
        return n, time.perf_counter() - t0


# --------------------------------------------------------------------------
L2_BYTES = 129e6  # GB300 L2


def timed_device_ms(fn, steps, stream, flush=None):
    """Device milliseconds of `steps` calls of fn on `stream`: one CUDA event
    pair around all of them, or, when `flush` (a tensor larger than L2) is
    given, one pair per call with a write of `flush` between the calls,
    outside the timed pairs, so that no call finds its inputs in L2."""
    import torch

    if flush is None:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)
    tot = 0.0
    for _ in range(steps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1)
    return tot


def l2_flush_buffer(input_bytes, device):
    """A 256 MB buffer to flush L2 between timed steps when a step's inputs
    fit in L2, else None."""
    import torch

    if input_bytes > L2_BYTES:
        return None
    return torch.empty(64 << 20, dtype=torch.float32, device=device)


def max_over_ranks(value, device):
    """The maximum of a per-rank float over the process group (itself when
    there is no group)."""
    import torch

    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def run_reference(args):
    rank, world, local = dist_info()
    if rank != 0:
        return 0
    wl = make_workload(args)
    kind = (None if wl.name in ("plain3d", "patches3d") else _ref_modules()) or "port"
    workers = os.cpu_count() or 1
    sample, desc = cpu_sample(wl, budget_s=6.0 * workers)
    for _ in range(args.warmup):
        time_cpu(wl, sample, kind, 1 if len(sample) == 1 else workers)
    tot_n, tot_t = 0, 0.0
    for _ in range(args.steps):
        n, t = time_cpu(wl, sample, kind, 1 if len(sample) == 1 else workers)
        tot_n += n
        tot_t += t
    value = tot_n / tot_t
    cores = 1 if len(sample) == 1 else workers
    line = {
        "impl": "reference", "metric": "output samples/sec (dip+SO filter)", "value": value,
        "unit": "samples/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot_t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, workloads.py)",
        "config": wl.config(),
        "cpu_baseline": {"value": value, "unit": "samples/s", "cores": cores, "kind": kind,
                         "sample": desc},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


PATCH = {"l": (64, 64), "s": (32, 32), "records": 16}


def measured_hbm_peak():
    """(GB/s, source): the measured copy bandwidth, else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return HBM_FALLBACK_GBS, "fallback"


def run_patch(args):
    """patch2d + patch2d_inv of the 2000 x 5000 DAS-like record in 64 x 64
    windows at stride 32 (the patch / DAS batching workflow's producer and
    consumer).  A step is one forward and one inverse pass over the record."""
    rank, world, local = dist_info()
    d = W.das2d(seed=args.seed + rank)
    n1, n2 = d.shape
    n = n1 * n2
    nrec = args.records or PATCH["records"]
    ls, ss = PATCH["l"], PATCH["s"]
    metric = "patched and reassembled samples/sec (patch2d + patch2d_inv)"
    config = {"workload": f"patch2d: {nrec} DAS-like records of {n1} x {n2} per step, windows "
                          f"{ls} at strides {ss}",
              "samples_per_step": nrec * n,
              "l2": "inputs larger than L2 (a record's patch matrix is 158 MB)"}
    if args.impl == "reference":
        if rank != 0:
            return 0
        from oracle import patch_oracle as P

        sub = d[:500, :1250]
        tt, m = 0.0, 0
        for k in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            P.patch_inv(P.patch(sub, ls, ss), sub.shape, ls, ss)
            if k >= args.warmup:
                tt += time.perf_counter() - t0
                m += sub.size
        value = m / tt
        desc = "500 x 1250 corner of the record, numpy restatement (oracle/patch_oracle.py)"
        print(json.dumps({
            "impl": "reference", "metric": metric, "value": value, "unit": "samples/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tt / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, workloads.py)",
            "config": dict(config),
            "cpu_baseline": {"value": value, "unit": "samples/s", "cores": 1, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}))
        return 0
    import torch

    if world > 1:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    import pyseistr_gb300 as ps
    from pyseistr_gb300 import _lib
    from pyseistr_gb300 import device as D

    _lib.load()
    dev = torch.device("cuda", local)
    a1 = torch.from_numpy(np.ascontiguousarray(d.reshape(-1, order="F"))).to(dev)
    npatch = D.patch_count((n1, n2), ls, ss)
    recs = [a1.clone() for _ in range(nrec)]  # distinct buffers: nothing stays in L2
    xs = [torch.empty((npatch, ls[0] * ls[1]), dtype=torch.float32, device=dev)
          for _ in range(nrec)]
    backs = [torch.empty_like(a1) for _ in range(nrec)]

    def step():
        for r in range(nrec):
            D.patch(recs[r], (n1, n2), ls, ss, out=xs[r])
            D.patch_inv(xs[r], (n1, n2), ls, ss, out=backs[r])

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        # untimed steps while the sampler starts (its period is 200 ms)
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 0.6:
            step()
            torch.cuda.synchronize()
        l0 = _lib.launch_count()
        ev0.record()
        for _ in range(args.steps):
            step()
        ev1.record()
        torch.cuda.synchronize()
    launches = _lib.launch_count() - l0
    ms = max_over_ranks(ev0.elapsed_time(ev1), dev) if world > 1 else ev0.elapsed_time(ev1)
    ms_step = ms / args.steps
    # per-kernel times: each direction moves 4 n + 4 npatch L algorithmic bytes
    # (average launch over all records of the timed steps, CUDA events)
    per = {}
    for name, fn in (("k_patch", lambda r: D.patch(recs[r], (n1, n2), ls, ss, out=xs[r])),
                     ("k_patch_inv",
                      lambda r: D.patch_inv(xs[r], (n1, n2), ls, ss, out=backs[r]))):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            for r in range(nrec):
                fn(r)
        e1.record()
        torch.cuda.synchronize()
        per[name] = e0.elapsed_time(e1) / (args.steps * nrec)
    dom = max(per, key=per.get)
    nbytes = 4 * n + 4 * npatch * ls[0] * ls[1]
    achieved = nbytes / (per[dom] / 1e3) / 1e9
    peak, peak_src = measured_hbm_peak()
    # end to end through the public API on host arrays
    t0 = time.perf_counter()
    for _ in range(args.steps):
        xh = ps.patch2d(d, *ls, *ss)
        bh = ps.patch2d_inv(xh, n1, n2, *ls, *ss)
    e2e = world * n / ((time.perf_counter() - t0) / args.steps)
    assert np.array_equal(bh, d)
    line = {
        "metric": metric, "value": world * nrec * n / (ms_step / 1e3), "unit": "samples/s",
        "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded, workloads.py)",
        "config": dict(config, parallelism=f"replicas x{world}"),
        "e2e": {"value": e2e, "unit": "samples/s",
                "h2d_bytes_per_step": 4 * n + 4 * xs[0].numel(),
                "d2h_bytes_per_step": 4 * xs[0].numel() + 4 * n},
        "gpu_launches": int(launches), "clocks": clk.summary(),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "peak_source": peak_src, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "kernel_ms": per,
                     "bytes_per_launch": nbytes},
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import patch_oracle as P

        sub = d[:500, :1250]
        t0 = time.perf_counter()
        P.patch_inv(P.patch(sub, ls, ss), sub.shape, ls, ss)
        line["cpu_baseline"] = {"value": sub.size / (time.perf_counter() - t0),
                                "unit": "samples/s", "cores": 1, "kind": "port",
                                "sample": "500 x 1250 corner, oracle/patch_oracle.py"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# the DAS demo's filter (demos/test_pyseistr_das.py:39): 2 kHz sampling,
# high cut at 200 Hz, 6 poles (3 per direction), zero phase
BANDPASS = {"dt": 0.0005, "flo": 0.0, "fhi": 200.0, "nplo": 6, "nphi": 6, "phase": 0,
            "records": 16}


def cpu_bandpass(d, bp, threads):
    """Seconds the oracle's C band-pass takes over the traces of `d`, split
    into `threads` column blocks run on as many host threads."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O

    args = (bp["dt"], bp["flo"], bp["fhi"], bp["nplo"], bp["nphi"], bp["phase"])
    edges = np.linspace(0, d.shape[1], threads + 1).astype(int)
    blocks = [np.asfortranarray(d[:, a:b]) for a, b in zip(edges[:-1], edges[1:]) if b > a]
    with ThreadPoolExecutor(len(blocks)) as pool:
        t0 = time.perf_counter()
        list(pool.map(lambda blk: O.bandpass(blk, *args), blocks))
        return time.perf_counter() - t0


def run_bandpass(args):
    """bandpassc of 2000 x 5000 DAS-like records with the DAS demo's filter
    (the step before the slope estimation in the DAS chain).  A step is 16
    records, each in its own buffer (640 MB of input, more than L2)."""
    rank, world, local = dist_info()
    d = W.das2d(seed=args.seed + rank)
    n1, n2 = d.shape
    n = n1 * n2
    bp = BANDPASS
    nrec = args.records or bp["records"]
    bpa = (bp["dt"], bp["flo"], bp["fhi"], bp["nplo"], bp["nphi"], bp["phase"])
    metric = "band-passed samples/sec (bandpassc, Butterworth, zero phase)"
    config = {"workload": f"bandpass2d: {nrec} DAS-like records of {n1} x {n2} per step, "
                          f"dt {bp['dt']} s, high cut {bp['fhi']} Hz, {bp['nphi']} poles, "
                          "zero phase",
              "samples_per_step": nrec * n,
              "l2": "inputs larger than L2 (16 distinct 40 MB records per step)",
              "e2e_input": "one column-major float32 host record per call"}
    threads = os.cpu_count() or 1
    if args.impl == "reference":
        if rank != 0:
            return 0
        tt, m = 0.0, 0
        for k in range(args.warmup + args.steps):
            t = cpu_bandpass(d, bp, threads)
            if k >= args.warmup:
                tt += t
                m += n
        value = m / tt
        desc = (f"one {n1} x {n2} record per step, oracle C restatement "
                f"(oracle/pwd_oracle.cpp) over {threads} threads")
        print(json.dumps({
            "impl": "reference", "metric": metric, "value": value, "unit": "samples/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tt / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, workloads.py)",
            "config": dict(config),
            "cpu_baseline": {"value": value, "unit": "samples/s", "cores": threads,
                             "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}))
        return 0
    import torch

    if world > 1:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    import pyseistr_gb300 as ps
    from pyseistr_gb300 import _lib
    from pyseistr_gb300 import device as D

    _lib.load()
    dev = torch.device("cuda", local)
    a1 = torch.from_numpy(np.ascontiguousarray(d.reshape(-1, order="F"))).to(dev)
    recs = [a1.clone() for _ in range(nrec)]
    outs = [torch.empty_like(a1) for _ in range(nrec)]
    shape = (n1, n2, 1)

    def step():
        for r in range(nrec):
            D.bandpass(recs[r], shape, *bpa, out=outs[r])

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 0.6:
            step()
            torch.cuda.synchronize()
        l0 = _lib.launch_count()
        ev0.record()
        for _ in range(args.steps):
            step()
        ev1.record()
        torch.cuda.synchronize()
    launches = _lib.launch_count() - l0
    ms = max_over_ranks(ev0.elapsed_time(ev1), dev) if world > 1 else ev0.elapsed_time(ev1)
    ms_step = ms / args.steps
    # one k_bandpass launch per record: the average over the timed steps
    per_launch_ms = ms_step / nrec
    nbytes = 8 * n  # each sample read once and written once
    achieved = nbytes / (per_launch_ms / 1e3) / 1e9
    peak, peak_src = measured_hbm_peak()
    # end to end through the public API on a host array, column-major as the
    # DAS demo reads its record (np.fromfile(...).reshape(..., order="F"))
    df = np.asfortranarray(d)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dh = ps.bandpassc(df, *bpa, verb=0)
    e2e = world * n / ((time.perf_counter() - t0) / args.steps)
    line = {
        "metric": metric, "value": world * nrec * n / (ms_step / 1e3), "unit": "samples/s",
        "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded, workloads.py)",
        "config": dict(config, parallelism=f"replicas x{world}"),
        "e2e": {"value": e2e, "unit": "samples/s", "h2d_bytes_per_step": 4 * n,
                "d2h_bytes_per_step": 4 * n},
        "gpu_launches": int(launches), "clocks": clk.summary(),
        "roofline": {"bound": "hbm", "kernel": "k_bandpass", "achieved": achieved,
                     "peak": peak, "peak_source": peak_src, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "kernel_ms": per_launch_ms,
                     "bytes_per_launch": nbytes,
                     "sweeps": 2 if bp["fhi"] > 0 and not bp["phase"] else 1},
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as O

        assert np.array_equal(dh, O.bandpass(d, *bpa))
        t, reps = 0.0, 0
        while t < 2.0:  # a bounded sample: whole records for about 2 s of wall time
            t += cpu_bandpass(d, bp, threads)
            reps += 1
        line["cpu_baseline"] = {"value": reps * n / t, "unit": "samples/s", "cores": threads,
                                "kind": "port",
                                "sample": f"{reps} passes over one {n1} x {n2} record, "
                                          "oracle/pwd_oracle.cpp"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


DASCOH = {"channels": 860, "w": 0.05, "nv": 100, "vmax": 0.005, "dt": 0.0005}


def run_das_fkcoh(args):
    """The DAS chain's last two steps on one detection window
    (demos/test_pyseistr_das_massive.py:198-200): fkdip(w = 0.05) and the
    adjoint coherence cohc over 100 linear slopes in [-0.005, 0.005] s per
    channel, on a 2000-sample x 860-channel window of the DAS-like record.
    Opt-in (--workload das_fkcoh); samples/s = window samples per step time."""
    rank, world, local = dist_info()
    p = DASCOH
    d = np.ascontiguousarray(W.das2d(seed=args.seed + rank)[:, :p["channels"]])
    n1, n2 = d.shape
    v = np.linspace(-p["vmax"], p["vmax"], p["nv"]).astype(np.float32)
    h = np.arange(n2, dtype=np.float32)
    metric = "window samples/sec (fkdip + cohc adjoint, DAS detection window)"
    config = {"workload": f"das_fkcoh: fkdip(w {p['w']}) + cohc(adjoint, linear, {p['nv']} "
                          f"slopes) of one {n1} x {n2} window per step",
              "samples_per_step": n1 * n2,
              "l2": "the window (6.9 MB) fits in L2: L2 flushed (a 256 MB write) between "
                    "timed steps"}
    if args.impl == "reference" or (rank == 0 and world == 1 and not args.no_cpu_baseline):
        from oracle import fk_oracle as F
        from oracle import oracle as O

        def cpu_step():
            t0 = time.perf_counter()
            F.fkdip(d, p["w"])
            O.Coherence()(d, v, h, 1, n1, p["dt"], -1)
            return time.perf_counter() - t0
    if args.impl == "reference":
        if rank != 0:
            return 0
        tt = 0.0
        for k in range(args.warmup + args.steps):
            t = cpu_step()
            if k >= args.warmup:
                tt += t
        value = args.steps * n1 * n2 / tt
        desc = "numpy fkdip restatement and the C coherence restatement, one core"
        print(json.dumps({
            "impl": "reference", "metric": metric, "value": value, "unit": "samples/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * tt / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, workloads.py)",
            "config": dict(config),
            "cpu_baseline": {"value": value, "unit": "samples/s", "cores": 1, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}))
        return 0
    import torch

    if world > 1:
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    import pyseistr_gb300 as ps
    from pyseistr_gb300 import _lib
    from pyseistr_gb300 import device as D

    _lib.load()
    dev = torch.device("cuda", local)
    x = torch.from_numpy(np.ascontiguousarray(d.reshape(-1, order="F"))).to(dev)
    vt, ht = torch.from_numpy(v).to(dev), torch.from_numpy(h).to(dev)
    fk_out = torch.empty(n1 * n2, dtype=torch.float64, device=dev)
    coh_out = torch.empty(n1 * p["nv"], dtype=torch.float32, device=dev)
    ws = torch.empty(_lib.load().pwd_fkdip_workspace_size(n1, n2, 0), dtype=torch.uint8,
                     device=dev)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]

    def step():
        D.fkdip(x, n1, n2, p["w"], out=fk_out, workspace=ws)
        D.coherence(x, vt, ht, 1, n1, p["dt"], -1, 0.0, out=coh_out)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    fk_ms = coh_ms = 0.0
    # the window fits in L2: flush it between the timed steps
    flush = l2_flush_buffer(4 * n1 * n2, dev)
    with ClockSampler(local) as clk:
        l0 = _lib.launch_count()
        t_all = 0.0
        for _ in range(args.steps):
            if flush is not None:
                flush.fill_(1.0)
            e[0].record()
            D.fkdip(x, n1, n2, p["w"], out=fk_out, workspace=ws)
            e[1].record()
            D.coherence(x, vt, ht, 1, n1, p["dt"], -1, 0.0, out=coh_out)
            e[2].record()
            torch.cuda.synchronize()
            fk_ms += e[0].elapsed_time(e[1])
            coh_ms += e[1].elapsed_time(e[2])
            t_all += e[0].elapsed_time(e[2])
    launches = _lib.launch_count() - l0
    ms = max_over_ranks(t_all, dev) if world > 1 else t_all
    ms_step = ms / args.steps
    # algorithmic bytes of the FK filter's Stockham passes (each reads and
    # writes its spectrum: the time FFTs over n2 traces of nf, the space
    # FFTs over nf/2 + 1 rows of nk, forward in complex64, inverse in
    # complex128) over the whole fkdip time (passes, transposes and mask)
    nf, nk = 1 << (n1 - 1).bit_length(), 1 << (n2 - 1).bit_length()
    nrow = nf // 2 + 1
    fk_bytes = (int(math.log2(nf)) * 2 * n2 * nf + int(math.log2(nk)) * 2 * nrow * nk) * (8 + 16)
    achieved = fk_bytes / (fk_ms / args.steps / 1e3) / 1e9
    peak, peak_src = measured_hbm_peak()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ps.cohc(d - ps.fkdip(d, p["w"]), {"h": h, "v": v, "nt": n1, "dt": p["dt"], "typ": 1})
    e2e = world * n1 * n2 / ((time.perf_counter() - t0) / args.steps)
    line = {
        "metric": metric, "value": world * n1 * n2 / (ms_step / 1e3), "unit": "samples/s",
        "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded, workloads.py)",
        "config": dict(config, parallelism=f"replicas x{world}", fk_ms=fk_ms / args.steps,
                       coh_ms=coh_ms / args.steps),
        "e2e": {"value": e2e, "unit": "samples/s", "h2d_bytes_per_step": 4 * n1 * n2,
                "d2h_bytes_per_step": 4 * n1 * p["nv"],
                "path": "fkdip then cohc on the difference, host arrays, as the DAS demo"},
        "gpu_launches": int(launches), "clocks": clk.summary(),
        "roofline": {"bound": "hbm", "kernel": "fkdip Stockham passes",
                     "achieved": achieved, "peak": peak, "peak_source": peak_src,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "bytes_per_call": fk_bytes,
                     "note": "the spectra (17-34 MB) stay in L2 between passes"},
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        t = cpu_step()
        line["cpu_baseline"] = {"value": n1 * n2 / t, "unit": "samples/s", "cores": 1,
                                "kind": "port",
                                "sample": "one window: oracle/fk_oracle.py and the coherence "
                                          "restatement of oracle/pwd_oracle.cpp"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# The other configurations, each measured by its own bench.py run (a fresh
# process: its own device state, workspaces and clock sampler) and reported
# inside the headline line; a leg that fails reports its error instead.
LEGS = [("das2d", "configuration 3"), ("patches3d", "configuration 5"),
        ("plain2d", "configuration 1"), ("plain3d", "configuration 2"),
        ("das_fkcoh", "DAS chain: fkdip + cohc")]
LEG_KEYS = ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "config", "e2e",
            "gpu_launches", "clocks", "roofline", "accuracy_vs_fp64", "plain_fp32", "spray_fp32",
            "cpu_baseline")


def run_legs(args):
    legs = {}
    for name, what in LEGS:
        cmd = [sys.executable, os.path.abspath(__file__), "--workload", name, "--steps",
               str(min(args.steps, 5)), "--warmup", "3", "--cpu-budget", "5", "--no-legs",
               "--seed", str(args.seed)]
        if args.no_cpu_baseline:
            cmd.append("--no-cpu-baseline")
        if args.no_tune:
            cmd.append("--no-tune")
        t0 = time.perf_counter()
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
            out = [l for l in r.stdout.splitlines() if l.startswith("{")]
            if r.returncode != 0 or not out:
                legs[name] = {"what": what, "error": (r.stderr or r.stdout)[-400:]}
                continue
            d = json.loads(out[-1])
            leg = {k: d[k] for k in LEG_KEYS if k in d}
            leg["what"] = what
            leg["wall_s"] = round(time.perf_counter() - t0, 1)
            legs[name] = leg
        except (subprocess.SubprocessError, ValueError) as e:
            legs[name] = {"what": what, "error": str(e)[-400:]}
    return legs


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["patch2d", "bandpass2d",
                                                               "das_fkcoh"], default="batch2d")
    ap.add_argument("--seed", type=int, default=2023)
    ap.add_argument("--sections", type=int, default=512,
                    help="sections of the batch2d workload, patches of patches3d (at most 64); "
                         "smaller counts for profiler captures")
    ap.add_argument("--precision", choices=["plain", "mixed"], default="mixed",
                    help="slope estimation arithmetic: plain (bit-faithful FP32) or mixed "
                         "(FP32 taps, fused convolution smoothing, FP64 reductions)")
    ap.add_argument("--no-graph", action="store_true",
                    help="launch the slope estimation kernel by kernel instead of replaying "
                         "its captured CUDA graph")
    ap.add_argument("--records", type=int, default=0,
                    help="records per step of the patch2d and bandpass2d workloads (default "
                         "16); smaller counts for profiler captures")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the autotuner (library defaults for the launch-shape knobs)")
    ap.add_argument("--no-legs", action="store_true",
                    help="batch2d only: skip the other configurations' legs of the line")
    ap.add_argument("--cpu-budget", type=float, default=15.0,
                    help="seconds of single-core CPU work for the cpu_baseline sample")
    args = ap.parse_args()

    if args.workload == "patch2d":
        return run_patch(args)
    if args.workload == "bandpass2d":
        return run_bandpass(args)
    if args.workload == "das_fkcoh":
        return run_das_fkcoh(args)
    if args.impl == "reference":
        return run_reference(args)

    import torch

    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from pyseistr_gb300 import _lib

    _lib.load()
    wl = make_workload(args, rank)
    dev = torch.device("cuda", local)
    dst = DeviceState(wl, dev)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    mixed = args.precision == "mixed"
    tuning = None
    if mixed and not args.no_tune and wl.name in ("batch2d", "das2d"):
        # the library's launch-shape knobs tuned on this workload (direct
        # launches: the knobs are read when the launch sequence is enqueued,
        # so before the graph capture), outside any timed region
        from pyseistr_gb300 import tune

        cache = os.environ.get("PWD_TUNE_CACHE") or os.path.join(
            os.path.expanduser("~"), ".cache", "pyseistr_gb300", "tune.json")
        os.makedirs(os.path.dirname(cache), exist_ok=True)
        timer = tune.gpu_step_timer(lambda: gpu_step(wl, dst, mixed), reps=2, warmup=1)
        t0 = time.perf_counter()
        choice, key = tune.autotune(dst.shapes, wl.filt["ns"], wl.dip["order"], wl.dip["rect"],
                                    True, timer, cache_path=cache)
        tune.apply(choice)
        tuning = {"class": key, "choice": choice,
                  "tuning_s": round(time.perf_counter() - t0, 1)}
    if not args.no_graph:
        dst.capture(wl, mixed)
    for _ in range(max(3, args.warmup)):
        gpu_step(wl, dst, mixed)
    torch.cuda.synchronize()

    # ---- timed region (device) ----
    stream = torch.cuda.current_stream()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    flush = l2_flush_buffer(4 * wl.samples(), dev)
    barrier()
    torch.cuda.synchronize()
    l0 = _lib.launch_count()
    with ClockSampler(local) as clk:
        dev_ms = timed_device_ms(lambda: gpu_step(wl, dst, mixed), args.steps, stream, flush)
    launches = _lib.launch_count() - l0
    if dst.graph is not None:  # replays do not pass through the launch counter
        launches += dst.graph.launches * args.steps
    barrier()
    ms = max_over_ranks(dev_ms, dev)
    ms_step = ms / args.steps
    value = world * wl.samples() / (ms_step / 1e3)

    # ---- per-family kernel time (CUDA events around each launch) over a
    # repetition of the timed steps ----
    torch.cuda.synchronize()
    graph, dst.graph = dst.graph, None  # per-launch events need the launches themselves
    with _lib.profile() as prof:
        for _ in range(args.steps):
            gpu_step(wl, dst, mixed)
        torch.cuda.synchronize()
    dst.graph = graph
    fam_ms = {f: v / args.steps for f, v in prof.ms.items()}
    fam_n = {f: v // args.steps for f, v in prof.launches.items()}
    # the HBM roofline is that of the largest HBM-bound family; the spray,
    # bound by FP32 issue and latency, has its own line (spray_fp32)
    dom = max((f for f in fam_ms if f != "spray"), key=lambda f: fam_ms[f])
    bpl = family_bytes(wl, fam_n, mixed)
    peak, peak_src = measured_hbm_peak()
    avg_launch_s = fam_ms[dom] / 1e3 / max(1, fam_n[dom])
    achieved = bpl.get(dom, 0.0) / avg_launch_s / 1e9 if avg_launch_s > 0 else 0.0
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            with open(tpath) as fh:
                tj = json.load(fh)
            ent = tj.get(wl.name, {}).get(args.precision, {}).get(dom)
            if ent:
                traffic = ent["bytes_per_sample"] * wl.samples()
        except (OSError, ValueError, KeyError):
            traffic = None

    # ---- end to end through the public API on host arrays ----
    host = None
    if wl.name in ("batch2d", "das2d", "patches3d"):  # pinned host inputs and outputs
        hd = torch.from_numpy(np.concatenate([s.reshape(-1, order="F") for s in wl.sections]))
        hd = hd.pin_memory()
        if wl.name == "patches3d":
            hm = torch.from_numpy(np.concatenate([m.reshape(-1, order="F") for m in wl.masks]))
            host = ((hd, hm.pin_memory()), torch.empty(hd.shape, dtype=torch.float32,
                                                       pin_memory=True))
        else:
            host = (hd, (torch.empty(hd.shape, dtype=torch.float32, pin_memory=True),
                         torch.empty(hd.shape, dtype=torch.float32, pin_memory=True)))
        api_step(wl, mixed, host)  # warm the workspaces of the packed path
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    h2d = d2h = 0
    for _ in range(args.steps):
        h2d, d2h = api_step(wl, mixed, host)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, dev)
    e2e = world * wl.samples() / e2e_s

    # accuracy of the timed path's outputs (still in place from the last step)
    acc = accuracy_vs_fp64(wl, dst, args.seed + rank) if rank == 0 else None
    plain = None
    if mixed:
        # the plain FP32 path on the same inputs: the mixed/plain ratio and
        # the distance between the two slope fields
        p_mixed = dst.p.clone()
        torch.cuda.synchronize()
        plain_ms = timed_device_ms(lambda: gpu_step(wl, dst, False), args.steps, stream,
                                   flush) / args.steps
        errs, k = [], 0
        for shp in dst.shapes:
            n = int(np.prod(shp))
            a, b = p_mixed[k:k + n].double(), dst.p[k:k + n].double()
            errs.append(float(torch.linalg.norm(a - b) / max(float(torch.linalg.norm(b)), 1e-30)))
            k += n
        plain = {"value": world * wl.samples() / (plain_ms / 1e3), "ms_per_step": plain_ms,
                 "speedup_mixed_vs_plain": plain_ms / ms_step,
                 "slopes_rel_l2_mixed_vs_plain_max_section": max(errs)}

    line = {
        "metric": "output samples/sec (dip+SO filter)", "value": value, "unit": "samples/s",
        "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, workloads.py)",
        "config": dict(wl.config(),
                       precision=("mixed: FP32 taps, convolution smoothing fused with the CG, "
                                  "FP64 reductions; filters plain FP32") if mixed
                       else "plain FP32 (bit-faithful to the reference)",
                       l2="inputs larger than L2 (129 MB)" if flush is None
                       else "inputs fit in L2: L2 flushed (a 256 MB write) between timed "
                            "steps, each step timed alone",
                       parallelism=f"replicas x{world}",
                       slope_launches="replay of the captured CUDA graph" if dst.graph
                       is not None else "kernel by kernel"),
        "e2e": {"value": e2e, "unit": "samples/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "roofline": {"bound": "hbm", "kernel_family": dom,
                     "largest_family": max(fam_ms, key=lambda f: fam_ms[f]),
                     "achieved": achieved, "peak": peak,
                     "peak_source": peak_src, "unit": "GB/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic,
                     "family_ms_per_step": fam_ms, "family_launches_per_step": fam_n},
    }
    if plain is not None:
        line["plain_fp32"] = plain
    if acc is not None:
        line["accuracy_vs_fp64"] = acc
    if tuning is not None:
        line["config"]["tuning"] = tuning
    if (rank == 0 and world == 1 and args.workload == "batch2d" and not args.no_legs
            and args.impl == "gb300"):
        torch.cuda.synchronize()
        line["legs"] = run_legs(args)
    if rank == 0 and fam_ms.get("spray", 0.0) > 0 and spray_flops_per_sample(wl):
        # the spray is bound by FP32 issue and latency, not by HBM: its
        # algorithmic flops per second against the measured FMA peak
        fpk = fp32_peak_tflops()
        ach = spray_flops_per_sample(wl) * wl.samples() / (fam_ms["spray"] / 1e3) / 1e12
        line["spray_fp32"] = {"bound": "fp32-issue", "achieved": ach, "peak": fpk,
                              "unit": "TFLOP/s", "frac": ach / fpk,
                              "flops_per_sample": spray_flops_per_sample(wl),
                              "peak_source": "measured: pwd_fp32_fma_probe"}
        # the same family against HBM: the DRAM bytes its launches move (the
        # ncu capture's per-sample traffic, profiles/traffic.json) per second
        try:
            with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
                ent = json.load(fh).get(wl.name, {}).get(args.precision, {}).get("spray")
        except (OSError, ValueError):
            ent = None
        if ent:
            gbs = (ent["bytes_per_sample"] * fam_n["spray"] * wl.samples()
                   / (fam_ms["spray"] / 1e3) / 1e9)
            line["spray_fp32"]["dram_traffic"] = {
                "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                "bytes_per_sample_per_launch": ent["bytes_per_sample"],
                "source": "profiles/traffic.json (ncu DRAM bytes of the 128-section case)"}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        kind = (None if wl.name in ("plain3d", "patches3d") else _ref_modules()) or "port"
        sample, desc = cpu_sample(wl, args.cpu_budget)
        n, t = time_cpu(wl, sample, kind, 1)
        line["cpu_baseline"] = {"value": n / t, "unit": "samples/s", "cores": 1, "kind": kind,
                                "sample": desc}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
