"""The reference arm of bench.py on the host: every step is one whole (here
fake) CPU solve timed as it runs, no warm-up solves, and no further solve is
started once the wall budget has passed; the line reports the steps timed."""
import io
import json
import os
import sys
import time
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class FakeSolve:
    threads = 3
    calls = 0

    def __init__(self):
        FakeSolve.calls = 0

    def solve(self):
        FakeSolve.calls += 1
        t = time.perf_counter()
        time.sleep(0.05)
        return {"seconds": time.perf_counter() - t + 0.001 * FakeSolve.calls, "eigenvalues": [1.0, 2.0]}

    def describe(self, r):
        return "a fake solve"


def run_arm(monkeypatch, argv):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(bench, "CpuSolve", FakeSolve)
    monkeypatch.setattr(bench, "load_fixture", lambda: None)
    monkeypatch.setattr(sys, "argv", ["bench.py"] + argv)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    out = io.StringIO()
    with redirect_stdout(out):
        bench.main()
    return json.loads(out.getvalue().strip().splitlines()[-1])


def test_reference_arm_stops_at_its_wall_budget(monkeypatch):
    line = run_arm(monkeypatch, ["--impl", "reference", "--steps", "20", "--warmup", "5", "--ref-budget", "0.3"])
    assert line["impl"] == "reference"
    assert 1 <= line["steps"] < 20 and line["steps"] == FakeSolve.calls     # no warm-up solve ran
    assert line["warmup"] == 0 and line["steps_requested"] == 20 and line["warmup_requested"] == 5
    assert len(line["steps_seconds"]) == line["steps"]
    ordered = sorted(line["steps_seconds"])
    assert line["value"] == pytest.approx(ordered[len(ordered) // 2] if len(ordered) % 2
                                          else 0.5 * (ordered[len(ordered) // 2 - 1] + ordered[len(ordered) // 2]))
    assert line["e2e"]["value"] == line["value"] and line["cpu_baseline"]["cores"] == 3


def test_reference_arm_times_every_requested_step_within_budget(monkeypatch):
    line = run_arm(monkeypatch, ["--impl", "reference", "--steps", "3", "--warmup", "2", "--ref-budget", "100"])
    assert line["steps"] == 3 and FakeSolve.calls == 3
