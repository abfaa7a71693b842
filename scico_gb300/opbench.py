"""Operator micro-benchmark: time one ctgpu operator on a benchmark workload.

    python -m scico_gb300.opbench --op proj2d_fwd --config c2 --reps 20

Ops: proj2d_fwd, proj2d_adj (one C-ABI call each, CUDA events per call),
admm (one fused ADMM-TV solve of --iters iterations).  Prints one JSON line
with the median time, interactions/s and the algorithmic-byte bandwidth
(4 B per pixel-view interaction + the output write).  Used for ncu captures
of single kernels.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import statistics

import torch

from . import _device, _lib, linop, workloads


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--op", default="proj2d_fwd", choices=["proj2d_fwd", "proj2d_adj", "admm"])
    ap.add_argument("--config", default="c2", choices=["c1", "c2"])
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--iters", type=int, default=2)
    ap.add_argument("--batch", type=int, default=1)
    a = ap.parse_args(argv)
    c = {"c1": workloads.C1, "c2": workloads.C2}[a.config]
    dev = _device.require_cuda()
    A = linop.XRayTransform2D((c.n, c.n), c.angles, det_count=c.det_count)
    g = A.geometry()
    img = torch.from_numpy(c.phantom()).to(dev).expand(a.batch, c.n, c.n).contiguous()
    sino = torch.empty((a.batch, c.n_views, c.det_count), device=dev)
    fwd_b, adj_b = A.workspace_bytes(a.batch)
    ws = _device.workspace(max(fwd_b, adj_b))
    s = torch.cuda.current_stream()
    if a.op == "proj2d_fwd":
        fn = lambda: _lib.call("ct_proj2d_fwd", ctypes.addressof(g), img.data_ptr(), sino.data_ptr(), a.batch,
                               ws.data_ptr(), ws.numel(), s.cuda_stream)
        alg = a.batch * (4.0 * c.interactions + 4.0 * c.n_views * c.det_count)
    elif a.op == "proj2d_adj":
        _lib.call("ct_proj2d_fwd", ctypes.addressof(g), img.data_ptr(), sino.data_ptr(), a.batch, ws.data_ptr(),
                  ws.numel(), s.cuda_stream)
        out = torch.empty_like(img)
        fn = lambda: _lib.call("ct_proj2d_adj", ctypes.addressof(g), sino.data_ptr(), out.data_ptr(), a.batch,
                               ws.data_ptr(), ws.numel(), s.cuda_stream)
        alg = a.batch * (4.0 * c.interactions + 4.0 * c.n * c.n)
    else:
        y = A(img[0].contiguous())
        desc = _lib.AdmmTvDesc(g, a.iters, c.cg_maxiter, c.cg_tol, 0.0, c.lam, 0.0, c.rho, 0.5, 1.0, 1)
        n = _lib.c_size_t()
        _lib.call("ct_admm_tv_workspace", ctypes.addressof(desc), ctypes.addressof(n))
        aws = _device.workspace(n.value)
        x = torch.zeros((c.n, c.n), device=dev)

        def fn():
            x.zero_()
            _lib.call("ct_admm_tv_solve", ctypes.addressof(desc), y.data_ptr(), x.data_ptr(), None, 0,
                      aws.data_ptr(), aws.numel(), s.cuda_stream)

        alg = 0.0
    for _ in range(a.warmup):
        fn()
    ts = []
    for _ in range(a.reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        fn()
        e1.record(s)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) / 1e3)
    t = statistics.median(ts)
    out = {"op": a.op, "config": a.config, "batch": a.batch, "median_s": t, "min_s": min(ts)}
    if alg:
        out.update(interactions_per_s=a.batch * c.interactions / t, alg_gbs=alg / t / 1e9)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
