"""Autotuner of the library's launch-shape knobs for a batched workload.

The kernels read a few tuning knobs from the environment at every call:

  PWD_CONV0_TMA    axis-0 tiles of the mixed CG staged by one bulk copy per
                   array (1, default) or element by element with cp.async (0)
  PWD_CG_STRIP     rows of an axis-1 strip of the mixed CG: 32, 64, 128
                   (default) or 256
  PWD_CONV1_PAIR   axis-1 passes of the mixed CG with one column per thread
                   (0, default) or two on packed FP32 pairs (1)
  PWD_SPRAY_BLOCK  threads per block of the spray's chain kernels: 32 or 64
                   (default)
  PWD_SPRAY_SPLIT  spray factor kernel: a thread per filter orientation (1),
                   per trace (0), or chosen by the wave count (unset)

and one switch that is not searched: PWD_CONV01=0 runs the cubes' axis-0
and axis-1 passes of gp as two kernels instead of one (the same bits).

None of them changes what is computed: the spray and the axis-0 staging
give the same bits whatever the setting, and the strip height and the
column pairing only change the order in which the mixed CG's FP64 dot
products are summed.

`autotune` times the workload's step (slope estimation and filter) under
candidate settings, one knob at a time from the defaults (coordinate
descent), keeps the fastest, and caches the choice per workload class: the
sections' median trace length and trace count rounded to powers of two,
their number rounded to a power of two, the filter radius, the order, the
smoothing radii and the precision mode.  `apply` sets a choice in the
environment.  The timer is a parameter, so the choice is deterministic
given the timings: the fastest candidate, the earlier one on ties.
"""
from __future__ import annotations

import json
import math
import os
from typing import Callable, Dict, List, Optional, Sequence, Tuple

KNOBS: Dict[str, List[Optional[str]]] = {
    "PWD_CONV0_TMA": ["1", "0"],
    "PWD_CG_STRIP": ["128", "64", "256", "32"],
    "PWD_CONV1_PAIR": ["0", "1"],
    "PWD_SPRAY_BLOCK": ["64", "32"],
    "PWD_SPRAY_SPLIT": [None, "1", "0"],
}
DEFAULTS = {k: v[0] for k, v in KNOBS.items()}


def _p2(x: float) -> int:
    return 1 << max(0, int(round(math.log2(max(1.0, x)))))


def workload_key(shapes: Sequence[Tuple[int, ...]], ns: int, order: int, rect, mixed: bool) -> str:
    """Class of a batch: what the launch shapes depend on."""
    n1 = sorted(s[0] for s in shapes)[len(shapes) // 2]
    n2 = sorted(s[1] for s in shapes)[len(shapes) // 2]
    return (f"n1~{_p2(n1)}/n2~{_p2(n2)}/nsec~{_p2(len(shapes))}/ns{ns}/o{order}/"
            f"r{'x'.join(str(int(r)) for r in rect)}/{'mixed' if mixed else 'plain'}")


def apply(choice: Dict[str, Optional[str]]) -> None:
    """Set a tuned choice in the environment (None: unset the knob)."""
    for k, v in choice.items():
        if v is None:
            os.environ.pop(k, None)
        else:
            os.environ[k] = str(v)


def search(time_step: Callable[[Dict[str, Optional[str]]], float],
           knobs: Dict[str, List[Optional[str]]] = KNOBS) -> Tuple[Dict[str, Optional[str]], Dict[str, float]]:
    """Coordinate descent over the knobs: for each knob in turn, every value
    with the others at their best so far; the fastest value stays (the
    earlier candidate on ties).  Returns (choice, timings by candidate)."""
    best = {k: v[0] for k, v in knobs.items()}
    seen: Dict[str, float] = {}

    def key(c):
        return ",".join(f"{k}={c[k]}" for k in sorted(c))

    def timed(c):
        kk = key(c)
        if kk not in seen:
            seen[kk] = float(time_step(dict(c)))
        return seen[kk]

    for name, values in knobs.items():
        t_best = timed(best)
        for v in values:
            cand = dict(best)
            cand[name] = v
            t = timed(cand)
            if t < t_best:
                t_best, best = t, cand
    return best, seen


def load_cache(path: str) -> dict:
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def autotune(shapes, ns, order, rect, mixed, time_step, cache_path: Optional[str] = None,
             retune: bool = False):
    """Tuned choice for a workload class, from the cache when present, else
    by `search` with `time_step(choice) -> seconds` (and stored)."""
    key = workload_key(shapes, ns, order, rect, mixed)
    cache = load_cache(cache_path) if cache_path else {}
    if not retune and key in cache:
        return cache[key]["choice"], key
    choice, seen = search(time_step)
    if cache_path:
        cache[key] = {"choice": choice, "timings_s": seen}
        tmp = cache_path + ".tmp"
        with open(tmp, "w") as fh:
            json.dump(cache, fh, indent=1, sort_keys=True)
        os.replace(tmp, cache_path)
    return choice, key


def gpu_step_timer(run: Callable[[], None], reps: int = 3, warmup: int = 1):
    """A time_step for `autotune`: sets the candidate, runs `run` warmup
    times, then times `reps` runs with CUDA events (median)."""
    import torch

    def time_step(choice):
        old = {k: os.environ.get(k) for k in choice}
        apply(choice)
        try:
            for _ in range(warmup):
                run()
            torch.cuda.synchronize()
            ts = []
            for _ in range(reps):
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record()
                run()
                b.record()
                torch.cuda.synchronize()
                ts.append(a.elapsed_time(b) / 1e3)
            ts.sort()
            return ts[len(ts) // 2]
        finally:
            apply(old)

    return time_step
