"""The autotuner's search and cache on the CPU, with recorded timings:
the choice is the fastest candidate (the earlier on ties), found by
coordinate descent from the defaults, and a cached choice is reused."""
import json

from pyseistr_gb300 import tune


def _timer(table, calls):
    def time_step(choice):
        calls.append(dict(choice))
        t = 1.0
        for k, v in choice.items():
            t += table.get((k, v), 0.0)
        return t
    return time_step


def test_search_picks_fastest_per_knob_and_prefers_earlier_on_ties():
    table = {("PWD_CG_STRIP", "64"): -0.2, ("PWD_CG_STRIP", "32"): -0.2,
             ("PWD_SPRAY_BLOCK", "32"): +0.1, ("PWD_CONV0_TMA", "0"): +0.05,
             ("PWD_SPRAY_SPLIT", "1"): -0.01}
    calls = []
    choice, seen = tune.search(_timer(table, calls))
    assert choice == {"PWD_CONV0_TMA": "1", "PWD_CG_STRIP": "64", "PWD_CONV1_PAIR": "0",
                      "PWD_SPRAY_BLOCK": "64", "PWD_SPRAY_SPLIT": "1"}
    # every distinct candidate timed once
    keys = [",".join(f"{k}={c[k]}" for k in sorted(c)) for c in calls]
    assert len(keys) == len(set(keys)) == len(seen)
    again, _ = tune.search(_timer(table, []))
    assert again == choice


def test_autotune_caches_per_workload_class(tmp_path):
    path = str(tmp_path / "tune.json")
    shapes = [(800, 300), (900, 350), (1000, 200)]
    calls = []
    t = _timer({("PWD_SPRAY_BLOCK", "32"): -0.5}, calls)
    c1, key = tune.autotune(shapes, 6, 2, (10, 10, 1), True, t, path)
    n = len(calls)
    c2, key2 = tune.autotune(shapes, 6, 2, (10, 10, 1), True, t, path)
    assert c1 == c2 and key == key2 and len(calls) == n
    assert c1["PWD_SPRAY_BLOCK"] == "32"
    with open(path) as fh:
        stored = json.load(fh)
    assert key in stored and stored[key]["choice"] == c1
    # another class is tuned afresh
    _, key3 = tune.autotune([(300, 60)] * 40, 6, 2, (10, 10, 1), True, t, path)
    assert key3 != key and len(calls) > n


def test_apply_sets_and_unsets(monkeypatch):
    monkeypatch.setenv("PWD_SPRAY_SPLIT", "1")
    tune.apply({"PWD_SPRAY_SPLIT": None, "PWD_CG_STRIP": "256"})
    import os

    assert "PWD_SPRAY_SPLIT" not in os.environ and os.environ["PWD_CG_STRIP"] == "256"
    tune.apply({"PWD_CG_STRIP": None})
    assert "PWD_CG_STRIP" not in os.environ
