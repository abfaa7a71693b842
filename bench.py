#!/usr/bin/env python
"""CT ADMM-TV benchmark: iterations/s of the 512x512 / 360-view / 725-bin
ADMM-TV reconstruction (lambda 0.005, rho 2, 100 iterations, CG <= 10).

A step is one complete 100-iteration ADMM-TV solve from x0 = 0 of a seeded
synthetic sinogram (20-ellipse phantom, 0.5%-of-peak Gaussian noise).

  value     iterations/s with the sinogram resident on the device: the fused
            native solver (ct_admm_tv_solve, each iteration one CUDA graph),
            CUDA events around each step, L2 flushed (256 MB write) before
            every step outside the events.
  e2e       the same metric through the public API (scico_gb300.optimize.ADMM
            with SquaredL2Loss / XRayTransform2D / FiniteDifference / L21Norm),
            with the sinogram copied from pinned host memory and the
            reconstruction copied back inside the timed region.
  roofline  the forward projector (dominant kernel) timed live with CUDA
            events: algorithmic bytes = 4 B per pixel-view interaction +
            the sinogram write, against the measured HBM copy bandwidth.
            That figure measures interaction throughput: the image and
            sinogram stay in L2, so the kernel is bound by instruction issue
            and shared memory, not DRAM; the measured DRAM bytes per call
            (ncu), their rate and the issue-slot figures are reported beside
            it.
  cpu_baseline  the C/OpenMP restatement of scico's path timed on all host
            cores for the same whole 100-iteration solve from x0 = 0.
  secondary the other workloads, each CUDA-event timed with its own clock
            samples: the 3D solve (256^3, 360 views), the 64 uneven scans
            solved in one batch call against per-scan loops, and the
            unrolled-CG training step (forward and backward).

``--config c5`` runs the 3D workload instead (256^3 volume, 360 views about
axis 0, L1 + L2,1 TV, 30 iterations, CG <= 8), with the same keys.

``--impl reference`` times that CPU restatement alone as the reference arm
(scico itself runs on JAX, which is not installable on these machines): the
same whole solve from x0 = 0, its iterations split over the --steps timed
steps (state carried from one step to the next), with the GPU solver's
precision policy (float64 CG dot products) so both arms run the same
algorithm; both lines report the CG steps their solve ran.
Multi-GPU (``--gpus N`` under torchrun): independent replicas, no collective
on the data path; value = all ranks' iterations / max time.
"""

from __future__ import annotations

import argparse
import datetime
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "CT ADMM-TV iters/s"
UNIT = "iter/s"
PEAKS = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM = 6800.0


def solve_projections(cg_its):
    """Projector applications (forward or adjoint calls that run) of one
    fused solve: A^T y once; A x and A^T A x in the first iteration and after
    every iteration whose CG moved x; one pair per CG step; A x in the
    epilogue when the last CG moved x.  The reference's loop applies 4 per
    iteration (A^T y, the CG start's pair, the objective's A x) and 2 per CG
    step."""
    n = 1 + (1 if cg_its and cg_its[-1] > 0 else 0)
    for i, k in enumerate(cg_its):
        n += (2 if i == 0 or cg_its[i - 1] > 0 else 0) + 2 * k
    return n


def solve_launches(cg_its, fast_forward=True):
    """Kernel launches of one fused solve whose iterations ran cg_its CG
    steps (CG_It from the solve's own itstat records).  Set-up: A^T y, its
    split sum, z/u init and the call reset (4); the itstat epilogue: rhs,
    forward strips and gather, residual, record (5).

    With the cooperative fast-forward kernels (the default on a GPU that
    runs cooperative launches; ct_solver_fast_forward): the graph's loop body
    starts at iteration 0 and after every iteration whose CG ran -- k_rhs,
    the projections of x (forward strips and gather, residual, adjoint: 4),
    the fast-forward CG start (1), which runs every following CG-free
    iteration inside its own launch, the CG steps of the iteration it hands
    back (forward strips and gather, adjoint, fused CG step = 4 each) and
    the z/u update (1).  Without them: per iteration k_rhs, the projections
    of x when CG moved x in the previous iteration or it is the first, the
    CG start, 6 launches per CG step (forward 2, adjoint, lhs, update,
    direction) and the z/u update."""
    n = 4 + 5
    m = len(cg_its)
    if not fast_forward:
        for i, k in enumerate(cg_its):
            dirty = i == 0 or cg_its[i - 1] > 0
            n += 1 + (4 if dirty else 0) + 1 + 6 * k + 1
        return n
    i = 0
    while i < m:
        n += 1 + 4 + 1 + 1
        j = i
        while j < m and cg_its[j] == 0:
            j += 1
        if j < m:
            n += 4 * cg_its[j]
        i = j + 1
    return n


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c5"],
                    help="c1/c2: 2D ADMM-TV (default c2); c5: 3D ADMM-TV, 256^3 x 360 views")
    ap.add_argument("--ref-precision", default="f64dots", choices=["f64dots", "f32"],
                    help="CPU restatement's CG scalars: float64 dot products (the GPU solver's policy, default) "
                         "or float32 (the reference's own)")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the secondary workloads (3D solve, batched scans, training step)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="use the planner's default projector schedule instead of measuring one first")
    return ap.parse_args()


def _workload(name):
    from scico_gb300 import workloads

    return {"c1": workloads.C1, "c2": workloads.C2, "c5": workloads.C5}[name]


def _config_json(c, name):
    return {
        "workload": f"ct_admm_tv_2d_{c.n}x{c.n}_{c.n_views}v_{c.det_count}b",
        "config": name,
        "image": c.n,
        "views": c.n_views,
        "det_count": c.det_count,
        "admm_iters_per_step": c.maxiter,
        "cg_maxiter": c.cg_maxiter,
        "lambda": c.lam,
        "rho": c.rho,
        "l2_flush": "256 MB write before every step",
        "parallelism": "replicas",
    }


def _hbm_peak():
    try:
        return float(json.loads(PEAKS.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


class ClockSampler:
    """nvidia-smi samples (SM clock, throttle reasons) during the timed region.

    nvidia-smi starts half a second before the region and samples every
    25 ms; only samples whose own timestamps fall inside the region count
    (all samples of the run are used, and said so, if none does)."""

    FIELDS = ["timestamp", "clocks.sm", "clocks.max.sm", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.t0 = self.t1 = 0.0

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={','.join(self.FIELDS)}",
                 "--format=csv,noheader,nounits", "-lms", "25"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.5)
        except Exception:
            self.proc = None
        self.t0 = time.time()
        return self

    def __exit__(self, *exc):
        self.t1 = time.time()
        self.result = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return False
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = []
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) != len(self.FIELDS):
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((ts, float(parts[1]), float(parts[2]), parts[3:]))
            except ValueError:
                continue
        inside = [r for r in rows if self.t0 <= r[0] <= self.t1]
        window = "timed region"
        if not inside:
            inside, window = rows, "whole run (no sample inside the timed region)"
        if inside:
            reasons = set()
            for r in inside:
                for name, val in zip(names, r[3]):
                    if val.lower().startswith("active"):
                        reasons.add(name)
            self.result = {"sm_mhz": statistics.median(r[1] for r in inside),
                           "sm_max_mhz": max(r[2] for r in inside), "reasons": sorted(reasons),
                           "samples": len(inside), "window": window}
        return False


# ---------------------------------------------------------------------------
# CPU restatement (baseline and reference arm)
# ---------------------------------------------------------------------------


def cpu_full_solve(c, threads: int, segments: int = 1, warmup: int = 0, dot64: bool = True):
    """The whole `c.maxiter`-iteration ADMM-TV solve of workload `c` from
    x0 = 0 on the C/OpenMP restatement, its iterations split into `segments`
    consecutive timed windows (the state carried from one to the next, so the
    windows together are exactly one solve).  `warmup` untimed single
    iterations of a throwaway solve come first.  Returns the per-window
    times, the iterations of each window, the solve's CG step counts, its
    final objective and the thread count used."""
    from oracle import ctref_c
    from scico_gb300 import workloads

    G = ctref_c.Geometry((c.n, c.n), c.angles, det_count=c.det_count)
    used = ctref_c.set_threads(threads)
    y = workloads.noisy(G.project(c.phantom()), c.noise, c.noise_seed)
    kw = dict(cg_maxiter=c.cg_maxiter, cg_tol=c.cg_tol, dot64=dot64)
    for _ in range(warmup):
        G.admm_tv(y, c.lam, c.rho, 1, **kw)
    bounds = np.linspace(0, c.maxiter, segments + 1).round().astype(int)
    state, times, n_its, stats = None, [], [], []
    for k in range(segments):
        n = int(bounds[k + 1] - bounds[k])
        n_its.append(n)
        if n == 0:
            times.append(0.0)
            continue
        t0 = time.perf_counter()
        x, z, u, it = G.admm_tv(y, c.lam, c.rho, n, state=state, **kw)
        times.append(time.perf_counter() - t0)
        state = (x, z, u)
        stats.append(it)
    it = np.concatenate(stats)
    return {"times": times, "iterations": n_its, "cg": [int(v) for v in it[:, 3]],
            "objective": float(it[-1, 0]), "threads": used}


def cpu_sample_3d(c, cg_steps: float, threads: int):
    """CPU estimate of one 3D ADMM-TV iteration: one forward and one adjoint
    of the C/OpenMP 3D projector on the workload, times the reference's
    K + 2 forward/adjoint pairs per iteration (K = CG steps).  Returns
    (iterations/s, threads, seconds timed, seconds per iteration)."""
    from oracle import ctref_c

    used = ctref_c.set_threads(threads)
    G = ctref_c.Geometry3D(c.shape, c.matrices().astype(np.float32), c.det_shape)
    x = c.phantom()
    t0 = time.perf_counter()
    y = G.project(x)
    t1 = time.perf_counter()
    G.back_project(y)
    t2 = time.perf_counter()
    per_iter = (cg_steps + 2.0) * (t2 - t0)
    return 1.0 / per_iter, used, t2 - t0, per_iter


def _config_json_3d(c, name):
    return {
        "workload": f"ct_admm_tv_3d_{c.n}^3_{c.n_views}v_{c.det_shape[0]}x{c.det_shape[1]}",
        "config": name, "volume": c.n, "views": c.n_views, "det_shape": list(c.det_shape),
        "admm_iters_per_step": c.maxiter, "cg_maxiter": c.cg_maxiter, "lambda_l1": c.lam_l1,
        "lambda_l21": c.lam_l21, "rho": c.rho, "l2_flush": "inputs (64 MB volume, 134 MB projections) plus a "
        "256 MB write before every step", "parallelism": "replicas",
    }


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import ctref_c

    if args.config == "c5":
        c = _workload("c5")
        threads = ctref_c.default_threads()
        vals, used, tsum = [], threads, 0.0
        for k in range(args.warmup + args.steps):
            v, used, dt, _ = cpu_sample_3d(c, c.cg_maxiter, threads)
            if k >= args.warmup:
                vals.append(v)
                tsum += dt
        value = statistics.median(vals)
        sample = (f"one forward and one adjoint of the C/OpenMP 3D projector per step on the {c.n}^3 x "
                  f"{c.n_views}-view workload, extrapolated to {c.cg_maxiter} + 2 pairs per ADMM iteration "
                  "(scico runs on JAX, not installable here)")
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tsum / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded 30-ellipsoid phantom)", "config": _config_json_3d(c, "c5"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": used, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}), flush=True)
        return 0
    c = _workload(args.config)
    dot64 = args.ref_precision == "f64dots"
    r = cpu_full_solve(c, ctref_c.default_threads(), segments=max(1, args.steps), warmup=args.warmup, dot64=dot64)
    total_t = sum(r["times"])
    value = c.maxiter / total_t
    pol = "float64 CG dot products (the GPU solver's precision policy)" if dot64 else \
        "float32 CG scalars (the reference's precision)"
    sample = (f"the whole {c.maxiter}-iteration ADMM-TV solve from x0 = 0 of the {c.n}x{c.n}/{c.n_views}/"
              f"{c.det_count} workload, split over the {args.steps} timed steps; C/OpenMP restatement of scico's "
              f"path with {pol}, every iteration as scico evaluates it (A^T y, itstat operator applications); "
              f"scico runs on JAX, not installable here")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / max(1, args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded 20-ellipse phantom, 0.5% Gaussian noise)",
        "config": _config_json(c, args.config),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": r["threads"], "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "solve_s": total_t, "cg_steps_total": int(sum(r["cg"])),
        "iterations_with_cg_steps": int(sum(1 for k in r["cg"] if k > 0)),
        "projector_applications": int(4 * c.maxiter + 2 * sum(r["cg"])), "final_objective": r["objective"],
        "ms_per_cg_step": 1e3 * total_t / max(1, int(sum(r["cg"]))),
        "ref_precision": args.ref_precision,
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# Multi-rank timing (one process per GPU, independent replicas)
# ---------------------------------------------------------------------------


def max_over_ranks(dist, t_local: float, device) -> float:
    """The largest of every rank's time (the job ends with its slowest rank);
    the rank's own time when not distributed."""
    if dist is None:
        return t_local
    import torch

    tt = torch.tensor([t_local], device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def whole_job_rate(units_per_rank: float, world: int, t_max: float) -> float:
    """Units all ranks processed per second of the slowest rank."""
    return units_per_rank * world / t_max


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------


def run_gpu(args):
    import ctypes

    import torch

    from scico_gb300 import _device, _lib, functional, linop, loss, workloads
    from scico_gb300.optimize import ADMM, LinearSubproblemSolver

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())
    c = _workload(args.config)

    # ---- workload (device) -------------------------------------------------
    A = linop.XRayTransform2D((c.n, c.n), c.angles, det_count=c.det_count)
    # projector launch schedules measured for this geometry and recorded
    # (ct_proj2d_autotune), once, before anything is timed
    schedule = A.autotune() if not args.no_autotune else A.schedule()
    x_gt = torch.from_numpy(c.phantom()).to(dev)
    y_clean = A(x_gt).cpu().numpy()
    y_host_np = workloads.noisy(y_clean, c.noise, c.noise_seed)
    y_host = torch.from_numpy(y_host_np).pin_memory()
    y_dev = y_host.to(dev)
    g = A.geometry()
    desc = _lib.AdmmTvDesc(g, c.maxiter, c.cg_maxiter, c.cg_tol, 0.0, c.lam, 0.0, c.rho, 0.5, 1.0, 1)
    nbytes = _lib.c_size_t()
    _lib.call("ct_admm_tv_workspace", ctypes.addressof(desc), ctypes.addressof(nbytes))
    ws = _device.workspace(nbytes.value)
    x = torch.zeros((c.n, c.n), device=dev)
    itstat = torch.zeros((c.maxiter, _lib.CT_ITSTAT_FIELDS), dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def solve():
        x.zero_()
        _lib.call("ct_admm_tv_solve", ctypes.addressof(desc), y_dev.data_ptr(), x.data_ptr(), itstat.data_ptr(),
                  0, ws.data_ptr(), ws.numel(), stream.cuda_stream)

    for _ in range(max(args.warmup, 3)):
        solve()
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- timed: device-resident --------------------------------------------
    barrier()
    times = []
    with ClockSampler(dev.index) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            solve()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
    barrier()
    t_max = max_over_ranks(dist, sum(times), dev)
    value = whole_job_rate(c.maxiter * args.steps, world, t_max)
    objective = float(itstat[c.maxiter - 1, _lib.CT_ITSTAT_OBJECTIVE])
    x_dev = x.clone()

    # ---- timed: end to end through the public API ----------------------------
    def e2e_step():
        yd = torch.empty((c.n_views, c.det_count), device=dev)
        yd.copy_(y_host, non_blocking=True)
        f = loss.SquaredL2Loss(y=yd, A=A)
        C = linop.FiniteDifference((c.n, c.n), append=0)
        s = ADMM(f=f, g_list=[c.lam * functional.L21Norm()], C_list=[C], rho_list=[c.rho], maxiter=c.maxiter,
                 subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": c.cg_tol, "maxiter": c.cg_maxiter}))
        xr = s.solve()
        return xr.cpu()

    for _ in range(2):
        e2e_step()
    barrier()
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xr = e2e_step()
        e2e_times.append(time.perf_counter() - t0)
    barrier()
    e2e_t = max_over_ranks(dist, sum(e2e_times), dev)
    e2e_value = whole_job_rate(c.maxiter * args.steps, world, e2e_t)
    e2e_dev_diff = float((xr.to(dev) - x_dev).norm() / x_dev.norm())

    # ---- roofline: the forward projector, live CUDA events ---------------------
    fwd_bytes, adj_bytes = A.workspace_bytes(1)
    pws = _device.workspace(max(fwd_bytes, adj_bytes))
    sino = torch.empty((c.n_views, c.det_count), device=dev)
    img = x_dev.clone()
    bp = torch.empty_like(img)

    def time_launches(fn, reps=20):
        for _ in range(3):
            fn()
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b) / 1e3)
        return statistics.median(ts)

    t_fwd = time_launches(lambda: _lib.call("ct_proj2d_fwd", ctypes.addressof(g), img.data_ptr(), sino.data_ptr(),
                                            1, pws.data_ptr(), pws.numel(), stream.cuda_stream))
    t_adj = time_launches(lambda: _lib.call("ct_proj2d_adj", ctypes.addressof(g), sino.data_ptr(), bp.data_ptr(),
                                            1, pws.data_ptr(), pws.numel(), stream.cuda_stream))
    inter = c.interactions
    alg_fwd = 4.0 * inter + 4.0 * c.n_views * c.det_count
    alg_adj = 4.0 * inter + 4.0 * c.n * c.n
    peak, peak_kind = _hbm_peak()
    achieved = alg_fwd / t_fwd / 1e9
    prof = _ncu_figures(f"proj2d_fwd_{args.config}")
    traffic = prof.get("dram_bytes_per_call")

    # ---- CPU baseline (rank 0, N = 1) -----------------------------------------
    cpu = None
    if rank == 0 and world == 1:
        try:
            from oracle import ctref_c

            r = cpu_full_solve(c, ctref_c.default_threads(), dot64=True)
            dt = sum(r["times"])
            cpu = {"value": c.maxiter / dt, "unit": UNIT, "cores": r["threads"], "kind": "port",
                   "sample": f"the whole {c.maxiter}-iteration solve from x0 = 0 ({dt:.1f} s, {sum(r['cg'])} CG "
                             "steps), C/OpenMP restatement of scico's path with float64 CG dot products",
                   "cg_steps_total": int(sum(r["cg"]))}
        except Exception as exc:  # the baseline is reported, not required
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {exc}"}

    cg_its = [int(v) for v in itstat[:, _lib.CT_ITSTAT_CG_ITERS].cpu().numpy()]
    launches_per_step = solve_launches(cg_its, bool(_lib.load().ct_solver_fast_forward()))
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded 20-ellipse phantom, 0.5% Gaussian noise)",
            "config": dict(_config_json(c, args.config), projector_schedule=schedule),
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": int(c.n_views * c.det_count * 4),
                    "d2h_bytes_per_step": int(c.n * c.n * 4),
                    "api": "scico_gb300.optimize.ADMM(...).solve()", "rel_diff_vs_value_path": e2e_dev_diff},
            "roofline": {"bound": "hbm", "kernel": "ct_proj2d_fwd", "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "algorithmic_bytes": alg_fwd, "launch_s": t_fwd,
                         "model": "4 B per pixel-view interaction + the sinogram write (a sweep that streams the "
                                  "image once per view); a measure of interaction throughput",
                         "interactions_per_s": inter / t_fwd,
                         "dram": None if traffic is None else {
                             "bytes_per_call": traffic, "gbs": traffic / t_fwd / 1e9,
                             "frac_of_hbm": traffic / t_fwd / 1e9 / peak},
                         "limiter": prof.get("limiter"),
                         "ncu": {k: v for k, v in prof.items() if k not in ("limiter", "dram_bytes_per_call")},
                         "adjoint": {"launch_s": t_adj, "achieved": alg_adj / t_adj / 1e9,
                                     "frac": alg_adj / t_adj / 1e9 / peak, "interactions_per_s": inter / t_adj}},
            "cpu_baseline": cpu,
            "clocks": clk.result,
            "gpu_launches": launches_per_step * args.steps,
            "final_objective": objective,
            "cg_steps_total": int(sum(cg_its)),
            "iterations_with_cg_steps": int(sum(1 for k in cg_its if k > 0)),
            "projector_applications": solve_projections(cg_its),
            "ms_per_cg_step": 1e3 * t_max / args.steps / max(1, int(sum(cg_its))),
        }
        if not args.no_secondary and world == 1:
            del ws, pws, flush
            torch.cuda.empty_cache()
            line["secondary"] = secondary(dev)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def _ncu_figures(name):
    """Figures of the last ncu capture of a kernel (profiles/<name>.json:
    DRAM bytes per call, issue activity, instructions per interaction, the
    limiter), or {} when none is committed."""
    f = ROOT / "profiles" / f"{name}.json"
    try:
        return json.loads(f.read_text())
    except (OSError, ValueError):
        return {}


def secondary(dev):
    """The other benchmark workloads at N = 1, each timed with CUDA events
    and its own clock samples: the 3D ADMM-TV solve (256^3, 360 views, 30
    iterations, CG <= 8), the CG-free proximal ADMM split of the same
    problem (native solver and generic loop) and the 3D forward projector;
    the 64 uneven scans (50
    iterations each) in one batch call against the fused per-scan graph
    loop, the per-scan loop with plain launches and the drop-in ADMM loop;
    the unrolled-CG training step (16 x 256^2, 5 blocks x CG 10)."""
    import torch

    from scico_gb300 import opbench, workloads

    out = {}
    peak, _ = _hbm_peak()
    with ClockSampler(dev.index) as clk:
        a3 = opbench.admm3d(dev, iters=workloads.C5.maxiter, warmup=1, reps=2)
    out["c5_admm_tv_3d"] = {"iters_per_s": a3["iters_per_s"], "s_per_solve": a3["median_s"],
                            "iterations": a3["iters"], "cg_steps_total": int(sum(a3["cg_steps"])),
                            "clocks": clk.result}
    with ClockSampler(dev.index) as clk:
        pd = opbench.padmm3d(dev, iters=20, warmup=1, reps=2)
    out["c5_padmm_tv_3d"] = {"fused_s_per_iter": pd["fused_s_per_iter"], "generic_s_per_iter": pd["generic_s_per_iter"],
                             "speedup": pd["speedup"], "iterations": pd["iters"], "clocks": clk.result}
    torch.cuda.empty_cache()
    with ClockSampler(dev.index) as clk:
        p3 = opbench.proj3d(dev, "fwd", warmup=2, reps=5)
    out["c5_proj3d_fwd"] = {"launch_s": p3["median_s"], "achieved_gbs": p3["alg_gbs"],
                            "frac": p3["alg_gbs"] / peak, "interactions_per_s": p3["interactions_per_s"],
                            "clocks": clk.result}
    torch.cuda.empty_cache()
    with ClockSampler(dev.index) as clk:
        b = opbench.c3(dev, iters=50, warmup=1, reps=2, autotune=True, plain=True)
    out["c3_batched_scans"] = {k: b[k] for k in ("scans", "iters", "batched_s", "scans_per_s", "looped_s",
                                                 "speedup", "looped_plain_launch_s", "speedup_vs_plain_launch",
                                                 "looped_generic_s", "speedup_vs_generic", "mean_cg_iters")}
    out["c3_batched_scans"]["clocks"] = clk.result
    torch.cuda.empty_cache()
    with ClockSampler(dev.index) as clk:
        m = opbench.modl(dev, warmup=2, reps=3)
    out["c4_unrolled_cg_training"] = {k: m[k] for k in ("batch", "forward_s", "backward_s",
                                                         "backward_over_forward", "images_per_s_train",
                                                         "peak_mem_gb")}
    out["c4_unrolled_cg_training"]["clocks"] = clk.result
    return out


def run_gpu_3d(args):
    """The 3D workload (C5): value through ct_admm_tv3d_solve, e2e through
    ADMM(...).solve() with XRayTransform3D, roofline of ct_proj3d_fwd."""
    import ctypes

    import torch

    from scico_gb300 import _device, _lib, functional, linop, loss, workloads
    from scico_gb300.optimize import ADMM, LinearSubproblemSolver

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())
    c = workloads.C5
    A = linop.XRayTransform3D(c.shape, c.matrices(), c.det_shape)
    x_gt = torch.from_numpy(c.phantom()).to(dev)
    y_dev = A(x_gt)
    gen = torch.Generator().manual_seed(c.noise_seed)
    y_dev = y_dev + c.noise * y_dev.abs().max() * torch.randn(y_dev.shape, generator=gen).to(dev)
    y_host = y_dev.cpu().pin_memory()
    g = A.geometry()
    desc = _lib.AdmmTv3dDesc(g, c.maxiter, c.cg_maxiter, c.cg_tol, 0.0, c.lam_l21, c.lam_l1, c.rho, 0.5, 1.0, 1)
    nbytes = _lib.c_size_t()
    _lib.call("ct_admm_tv3d_workspace", ctypes.addressof(desc), ctypes.addressof(nbytes))
    ws = _device.workspace(nbytes.value)
    x = torch.zeros(c.shape, device=dev)
    itstat = torch.zeros((c.maxiter, _lib.CT_ITSTAT_FIELDS), dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def solve():
        x.zero_()
        _lib.call("ct_admm_tv3d_solve", ctypes.addressof(desc), y_dev.data_ptr(), x.data_ptr(), itstat.data_ptr(),
                  0, ws.data_ptr(), ws.numel(), stream.cuda_stream)

    for _ in range(max(args.warmup, 3)):
        solve()
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    barrier()
    times = []
    with ClockSampler(dev.index) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            solve()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
    barrier()
    t_max = max_over_ranks(dist, sum(times), dev)
    value = whole_job_rate(c.maxiter * args.steps, world, t_max)
    cg_its = [int(v) for v in itstat[:, _lib.CT_ITSTAT_CG_ITERS].cpu().numpy()]
    x_dev = x.clone()

    def e2e_step():
        yd = torch.empty(A.output_shape, device=dev)
        yd.copy_(y_host, non_blocking=True)
        f = loss.SquaredL2Loss(y=yd, A=A)
        C = linop.FiniteDifference(c.shape, append=0)
        s = ADMM(f=f, g_list=[c.lam_l21 * functional.L21Norm(), c.lam_l1 * functional.L1Norm()], C_list=[C, C],
                 rho_list=[c.rho] * 2, maxiter=c.maxiter,
                 subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": c.cg_tol, "maxiter": c.cg_maxiter}))
        return s.solve().cpu()

    e2e_step()
    barrier()
    e2e_t = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xr = e2e_step()
        e2e_t += time.perf_counter() - t0
    barrier()
    e2e_t = max_over_ranks(dist, e2e_t, dev)
    e2e_value = whole_job_rate(c.maxiter * args.steps, world, e2e_t)
    e2e_diff = float((xr.to(dev) - x_dev).norm() / x_dev.norm())

    # roofline: the 3D forward projector, live CUDA events
    fwd_b, _ = A.workspace_bytes(1)
    pws = _device.workspace(fwd_b)
    proj = torch.empty(A.output_shape, device=dev)
    for _ in range(3):
        _lib.call("ct_proj3d_fwd", ctypes.addressof(g), x_dev.data_ptr(), proj.data_ptr(), 1, pws.data_ptr(),
                  pws.numel(), stream.cuda_stream)
    ts = []
    for _ in range(10):
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        _lib.call("ct_proj3d_fwd", ctypes.addressof(g), x_dev.data_ptr(), proj.data_ptr(), 1, pws.data_ptr(),
                  pws.numel(), stream.cuda_stream)
        a1.record(stream)
        a1.synchronize()
        ts.append(a0.elapsed_time(a1) / 1e3)
    t_fwd = statistics.median(ts)
    inter = c.interactions
    alg = 4.0 * inter + 4.0 * proj.numel()
    peak, peak_kind = _hbm_peak()
    achieved = alg / t_fwd / 1e9

    cpu = None
    if rank == 0 and world == 1:
        try:
            from oracle import ctref_c

            k = float(np.mean(cg_its)) if cg_its else c.cg_maxiter
            v, used, dt, per_iter = cpu_sample_3d(c, k, ctref_c.default_threads())
            cpu = {"value": v, "unit": UNIT, "cores": used, "kind": "port",
                   "sample": f"one forward + one adjoint of the C/OpenMP 3D projector ({dt:.1f} s), extrapolated "
                             f"to {k:.1f} + 2 pairs per ADMM iteration ({per_iter:.1f} s per iteration)"}
        except Exception as exc:
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": f"failed: {exc}"}
    # as the 2D solver (the 3D forward is also 2 kernels, the adjoint 1)
    launches_per_step = solve_launches(cg_its, bool(_lib.load().ct_solver_fast_forward()))
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded 30-ellipsoid phantom, 1% Gaussian noise)",
            "config": _config_json_3d(c, "c5"),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(proj.numel() * 4),
                    "d2h_bytes_per_step": int(x.numel() * 4), "api": "scico_gb300.optimize.ADMM(...).solve()",
                    "rel_diff_vs_value_path": e2e_diff},
            "roofline": {"bound": "hbm", "kernel": "ct_proj3d_fwd", "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                         "algorithmic_bytes": alg, "launch_s": t_fwd, "interactions_per_s": inter / t_fwd},
            "cpu_baseline": cpu, "clocks": clk.result, "gpu_launches": launches_per_step * args.steps,
            "cg_steps_per_iteration": cg_its,
        }), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    args = _args()
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "c5":
        return run_gpu_3d(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
