"""bench.py's clock sampler on a stand-in nvidia-smi (a script printing one CSV line every 20 ms):
started ahead of the timed region it keeps only the samples that arrived inside the region, reads
the throttle reasons, and its child process does not outlive the region.  No GPU."""
import importlib.util
import os
import stat
import sys
import time

import pytest

from conftest import ROOT

FAKE = """#!{py}
import sys, time
i = 0
while True:
    reason = "Active" if i % 2 else "Not Active"
    print(f"0, {{1900 + i}}, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, {{reason}}", flush=True)
    i += 1
    time.sleep(0.02)
"""


@pytest.fixture
def bench(tmp_path, monkeypatch):
    exe = tmp_path / "nvidia-smi"
    exe.write_text(FAKE.format(py=sys.executable))
    exe.chmod(exe.stat().st_mode | stat.S_IEXEC)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_samples_come_from_the_timed_region_only(bench):
    pytest.importorskip("torch")
    clk = bench.ClockSampler(0).start()
    time.sleep(0.5)                               # the warm-up: samples here are not the region's
    with clk:
        time.sleep(0.3)
    s = clk.summary()
    assert s is not None and 5 <= s["samples"] <= 25, s
    assert s["sm_max_mhz"] == 2070.0
    clock = lambda ln: float(ln.split(",")[1])  # noqa: E731  (the fake's clock rises line by line)
    before = [clock(ln) for t, ln in clk.arrived if t < clk.window[0]]
    assert before and min(clock(ln) for ln in clk.lines) > max(before)   # the warm-up's lines were left out
    assert s["reasons"] == ["sw_power_cap"]
    assert clk.p.poll() is not None               # the sampler process ended with the region


def test_no_sampler_no_clocks(bench, monkeypatch):
    pytest.importorskip("torch")
    monkeypatch.setenv("PATH", "/nonexistent")
    with bench.ClockSampler(0) as clk:
        pass
    assert clk.summary() is None
