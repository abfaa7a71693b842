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


def _rank_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(REPO))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t_max = bench.max_over_ranks(dist, 1.0 + 0.5 * rank, "cpu")
        out.put((rank, t_max, bench.whole_job_rate(100, world, t_max)))
    finally:
        dist.destroy_process_group()


def _free_port():
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_max_over_ranks_gloo_world2():
    """Two replicas on gloo: every rank gets the slowest rank's time, and the
    whole-job rate counts both ranks' units."""
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[1] for g in got] == [1.5, 1.5]
    assert all(abs(g[2] - 200 / 1.5) < 1e-9 for g in got)


def test_single_process_rate():
    sys.path.insert(0, str(REPO))
    import bench

    assert bench.max_over_ranks(None, 2.0, "cpu") == 2.0
    assert bench.whole_job_rate(100, 1, 2.0) == 50.0


def test_reference_arm_nonzero_rank_exits_quietly():
    """Under torchrun only rank 0 runs the reference arm; the others exit 0
    without output."""
    import subprocess

    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_launch_and_projection_accounting():
    """bench.solve_launches / solve_projections from a solve's CG step
    counts: set-up 4 + epilogue 5; with the cooperative kernels a pass of the
    graph's loop body (iteration 0 and every iteration after one whose CG
    ran) is k_rhs, 4 projection launches, the fast-forward CG start and the
    z/u update, plus 4 launches per CG step of the iteration it hands back
    (the CG-free iterations in between run inside the fast-forward launch);
    without them every iteration launches its own kernels, 6 per CG step."""
    import bench

    cg = [10, 10, 7, 0, 0, 5, 0, 0]
    assert bench.solve_launches(cg, True) == 9 + (7 + 40) + (7 + 40) + (7 + 28) + (7 + 20) + 7
    per_iter = [1 + (4 if i == 0 or cg[i - 1] > 0 else 0) + 1 + 6 * k + 1 for i, k in enumerate(cg)]
    assert bench.solve_launches(cg, False) == 9 + sum(per_iter)
    assert bench.solve_launches([0, 0, 0], True) == 9 + 7  # one pass: the CG start runs all three
    # A^T y, the epilogue's A x (the last CG moved x), a pair per CG step and
    # per iteration after a CG step
    assert bench.solve_projections([3, 0, 2]) == 1 + 1 + (2 + 6) + (2 + 0) + (0 + 4)
