"""Host logic of bench.py that needs no GPU: the clock sampler, fed by a
stand-in nvidia-smi that prints timestamped samples."""

import os
import stat
import sys
import time
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]

FAKE_SMI = """#!{python}
import datetime, sys, time
rate = float(sys.argv[sys.argv.index("-lms") + 1]) / 1000.0
for i in range(2000):
    now = datetime.datetime.now().strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    clock = 1800 if i % 2 else 2070
    print(f"{{now}}, {{clock}}, 2070, Not Active, Not Active, Not Active, Active", flush=True)
    time.sleep(rate)
"""


@pytest.fixture
def fake_smi(tmp_path, monkeypatch):
    exe = tmp_path / "nvidia-smi"
    exe.write_text(FAKE_SMI.format(python=sys.executable))
    exe.chmod(exe.stat().st_mode | stat.S_IEXEC)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    return exe


def test_clock_sampler_keeps_timed_region(fake_smi):
    sys.path.insert(0, str(REPO))
    import bench

    with bench.ClockSampler(0) as clk:
        time.sleep(0.3)
    r = clk.result
    assert r["window"] == "timed region"
    assert 4 <= r["samples"] <= 20  # ~25 ms sampling over 0.3 s
    assert r["sm_max_mhz"] == 2070.0
    assert r["sm_mhz"] in (1800.0, 1935.0, 2070.0)
    assert r["reasons"] == ["sw_power_cap"]


def test_clock_sampler_without_nvidia_smi(tmp_path, monkeypatch):
    sys.path.insert(0, str(REPO))
    import bench

    monkeypatch.setenv("PATH", str(tmp_path))
    with bench.ClockSampler(0) as clk:
        pass
    assert clk.result["samples"] == 0 and clk.result["sm_mhz"] is None
