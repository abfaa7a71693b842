"""Operator micro-benchmark: time one ctgpu operator on a benchmark workload.

    python -m scico_gb300.opbench --op proj2d_fwd --config c2 --reps 20

Ops: proj2d_fwd, proj2d_adj (one C-ABI call each, CUDA events per call),
admm (one fused ADMM-TV solve of --iters iterations), proj3d_fwd and
proj3d_adj (the 256^3, 360-view workload; --views N takes the first N views,
--general runs the GENERAL kernels on it), admm3d (one fused 3D ADMM-TV
solve of --iters iterations on that workload), padmm3d (--iters proximal ADMM
iterations of the CG-free 3D TV split, native solver and generic loop),
modl (one MoDL training
step, forward and backward, on the 16-slice batch), c3 (the 64 uneven scans
solved in one batch call and in a loop).  Prints one JSON line
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

from . import _device, _lib, functional, linop, loss, workloads
from .optimize import ADMM, LinearSubproblemSolver


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--op", default="proj2d_fwd",
                    choices=["proj2d_fwd", "proj2d_adj", "admm", "proj3d_fwd", "proj3d_adj", "admm3d", "padmm3d",
                             "modl", "c3"])
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c5"])
    ap.add_argument("--views", type=int, default=0, help="proj3d: first N views of the workload (0 = all)")
    ap.add_argument("--recompute", action="store_true", help="modl: recompute CG steps in the backward pass")
    ap.add_argument("--cudnn-search", type=int, default=1, choices=[0, 1],
                    help="modl: 1 = cuDNN picks convolution algorithms by measuring them (as XLA autotunes its "
                         "convolutions), 0 = cuDNN's heuristics")
    ap.add_argument("--streams", type=int, default=0, help="c3: internal streams of the batch solve (0 = auto)")
    ap.add_argument("--autotune", action="store_true",
                    help="c3, modl: measure and record projector schedules (ct_proj2d_autotune) before timing")
    ap.add_argument("--plain", action="store_true",
                    help="c3: also time the per-scan loops without graphs (fused solver with plain launches, "
                         "and scico_gb300.optimize.ADMM on the drop-in operators)")
    ap.add_argument("--general", action="store_true",
                    help="proj3d: run the GENERAL kernels on the workload's geometry")
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--iters", type=int, default=2)
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--graph", type=int, default=1, choices=[0, 1],
                    help="admm: 1 = one CUDA graph per iteration (the default solver), 0 = plain launches")
    a = ap.parse_args(argv)
    dev = _device.require_cuda()
    if a.op.startswith("proj3d"):
        return print(json.dumps(proj3d(dev, a.op[7:], a.views, a.general, a.warmup, a.reps)))
    if a.op == "admm3d":
        return print(json.dumps(admm3d(dev, a.iters, a.warmup, a.reps, a.graph)))
    if a.op == "padmm3d":
        return print(json.dumps(padmm3d(dev, a.iters, a.warmup, a.reps)))
    if a.op == "modl":
        return print(json.dumps(modl(dev, a.warmup, a.reps, a.recompute, a.autotune, bool(a.cudnn_search))))
    if a.op == "c3":
        return print(json.dumps(c3(dev, a.iters, a.warmup, a.reps, a.streams, a.autotune, a.plain)))
    c = {"c1": workloads.C1, "c2": workloads.C2}[a.config]
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
        desc = _lib.AdmmTvDesc(g, a.iters, c.cg_maxiter, c.cg_tol, 0.0, c.lam, 0.0, c.rho, 0.5, 1.0, a.graph)
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


def _time(fn, s, warmup, reps):
    for _ in range(warmup):
        fn()
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        fn()
        e1.record(s)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) / 1e3)
    return statistics.median(ts), min(ts)


def proj3d(dev, which="fwd", views=0, general=False, warmup=3, reps=20):
    """3D projector on the 256^3 / 360-view workload (random volume: the
    projector's time does not depend on the values); which = "fwd" or "adj",
    views = first N views (0 = all), general = run the GENERAL kernels."""
    c = workloads.C5
    M = c.matrices()
    if views:
        M = M[:views]
    A = linop.XRayTransform3D(c.shape, M, c.det_shape)
    g = A.geometry()
    if general:
        g.kind = _lib.CT_PROJ3D_GENERAL
    nv = len(M)
    vol = torch.rand(c.shape, generator=torch.Generator().manual_seed(0)).to(dev)
    proj = torch.empty(A.output_shape, device=dev)
    fwd_b, adj_b = A.workspace_bytes()
    ws = _device.workspace(max(fwd_b, adj_b))
    s = torch.cuda.current_stream()
    if which == "fwd":
        fn = lambda: _lib.call("ct_proj3d_fwd", ctypes.addressof(g), vol.data_ptr(), proj.data_ptr(), 1,
                               ws.data_ptr(), ws.numel(), s.cuda_stream)
        out_bytes = 4.0 * proj.numel()
    else:
        proj.copy_(torch.rand(A.output_shape, generator=torch.Generator().manual_seed(1)))
        out = torch.empty_like(vol)
        fn = lambda: _lib.call("ct_proj3d_adj", ctypes.addressof(g), proj.data_ptr(), out.data_ptr(), 1,
                               ws.data_ptr(), ws.numel(), s.cuda_stream)
        out_bytes = 4.0 * vol.numel()
    t, tmin = _time(fn, s, warmup, reps)
    inter = c.n**3 * nv
    return {"op": "proj3d_" + which, "config": "c5", "views": nv, "kind": "general" if general else A.kind,
            "median_s": t, "min_s": tmin, "interactions_per_s": inter / t,
            "alg_gbs": (4.0 * inter + out_bytes) / t / 1e9}


def admm3d(dev, iters=2, warmup=3, reps=20, graph=1):
    """`iters` fused 3D ADMM-TV iterations on the 256^3, 360-view workload
    (L1 + L2,1 on one FD, rho 1, CG <= 8), CUDA events per solve.  Reports
    seconds per iteration and the CG steps taken."""
    c = workloads.C5
    A = linop.XRayTransform3D(c.shape, c.matrices(), c.det_shape)
    x_gt = torch.from_numpy(workloads.random_ellipsoids(c.n, c.n_ellipsoids, c.phantom_seed)).to(dev)
    y = A(x_gt)
    y = y + c.noise * y.abs().max() * torch.randn(y.shape, generator=torch.Generator().manual_seed(c.noise_seed)).to(dev)
    g = A.geometry()
    desc = _lib.AdmmTv3dDesc(g, iters, c.cg_maxiter, c.cg_tol, 0.0, c.lam_l21, c.lam_l1, c.rho, 0.5, 1.0, graph)
    n = _lib.c_size_t()
    _lib.call("ct_admm_tv3d_workspace", ctypes.addressof(desc), ctypes.addressof(n))
    ws = _device.workspace(n.value)
    x = torch.zeros(c.shape, device=dev)
    itstat = torch.zeros((iters, _lib.CT_ITSTAT_FIELDS), dtype=torch.float64, device=dev)
    s = torch.cuda.current_stream()

    def fn():
        x.zero_()
        _lib.call("ct_admm_tv3d_solve", ctypes.addressof(desc), y.data_ptr(), x.data_ptr(), itstat.data_ptr(), 0,
                  ws.data_ptr(), ws.numel(), s.cuda_stream)

    t, tmin = _time(fn, s, warmup, reps)
    cg = itstat[:, _lib.CT_ITSTAT_CG_ITERS].cpu().numpy()
    return {"op": "admm3d", "config": "c5", "iters": iters, "graph": graph, "median_s": t,
            "s_per_iter": t / iters, "iters_per_s": iters / t, "cg_steps": [int(v) for v in cg],
            "objective": [float(v) for v in itstat[:, _lib.CT_ITSTAT_OBJECTIVE].cpu().numpy()]}


def padmm3d(dev, iters=20, warmup=1, reps=2, generic=True):
    """Proximal ADMM with the split of the reference's ct_3d_tv_padmm example
    (A = (C; alpha D), B = -I, g = 1/2 ||y - z0||^2 + (lam / alpha) ||z1||_{2,1};
    alpha 1e2, lam 2, rho 5e-3) on the 256^3 / 360-view workload: `iters`
    iterations through the native solver (one graph replayed per iteration)
    and, with `generic`, through the generic step loop, CUDA events around
    each solve."""
    from .functional import L21Norm, SeparableFunctional, ZeroFunctional
    from .loss import SquaredL2Loss as L2
    from .optimize import ProximalADMM

    c = workloads.C5
    C = linop.XRayTransform3D(c.shape, c.matrices(), c.det_shape)
    x_gt = torch.from_numpy(c.phantom()).to(dev)
    y = C(x_gt)
    y = y + c.noise * y.abs().max() * torch.randn(y.shape, generator=torch.Generator().manual_seed(c.noise_seed)).to(dev)
    alpha, lam, rho = 1e2, 2.0, 5e-3
    D = linop.FiniteDifference(c.shape, append=0)
    A = linop.VerticalStack((C, alpha * D))
    mu, nu = ProximalADMM.estimate_parameters(A, maxiter=20, seed=0)
    s = torch.cuda.current_stream()
    out = {"op": "padmm3d", "config": "c5", "iters": iters, "mu": mu, "nu": nu}

    def make(fused):
        g = SeparableFunctional((L2(y=y), (lam / alpha) * L21Norm()))
        return ProximalADMM(f=ZeroFunctional(), g=g, A=A, rho=rho, mu=mu, nu=nu, maxiter=iters, fused=fused)

    for name, fused in (("fused", True), ("generic", False)):
        if name == "generic" and not generic:
            continue
        t, _ = _time(lambda: make(fused).solve(), s, warmup, reps)
        out[name + "_s_per_iter"] = t / iters
    if generic:
        out["speedup"] = out["generic_s_per_iter"] / out["fused_s_per_iter"]
    return out


def modl(dev, warmup=3, reps=20, recompute=False, autotune=False, cudnn_search=True):
    """One MoDL training step on the C4 batch (16 x 256^2, 180 views; 5
    blocks of CG(10) on A^T A + lmbda I, 3-layer 32-filter ResNet): forward
    with the MSE loss, then backward, each timed with CUDA events.
    Convolutions in full float32 (TF32 off)."""
    from . import inverse

    torch.backends.cudnn.allow_tf32 = False
    torch.backends.cuda.matmul.allow_tf32 = False
    # cuDNN's measured algorithm choice (the counterpart of XLA's convolution
    # autotuning); its heuristics pick FFT-tiled backward convolutions here
    torch.backends.cudnn.benchmark = cudnn_search
    c = workloads.C4
    H = linop.XRayTransform2D((c.n, c.n), c.angles, det_count=c.det_count)
    schedule = H.autotune(batch=c.batch, reps=5) if autotune else H.schedule(batch=c.batch)
    x_gt = torch.from_numpy(c.phantoms()).to(dev)
    y = H.project(x_gt)
    y = y + c.noise * y.abs().max() * torch.randn(y.shape, generator=torch.Generator().manual_seed(c.phantom_seed)).to(dev)
    torch.manual_seed(c.weight_seed)
    net = inverse.MoDLNet(H, depth=c.depth, channels=1, num_filters=c.num_filters, block_depth=c.block_depth,
                          lmbda_ini=c.lmbda_ini, cg_iter=c.cg_iter, cg_recompute=recompute).to(dev)
    s = torch.cuda.current_stream()
    fts, bts = [], []
    for k in range(warmup + reps):
        net.zero_grad(set_to_none=True)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(s)
        loss = ((net(y) - x_gt) ** 2).mean()
        e1.record(s)
        loss.backward()
        e2.record(s)
        e2.synchronize()
        if k >= warmup:
            fts.append(e0.elapsed_time(e1) / 1e3)
            bts.append(e1.elapsed_time(e2) / 1e3)
    tf, tb = statistics.median(fts), statistics.median(bts)
    n_proj = c.batch * (c.depth * (c.cg_iter + 1) * 2 + 1)  # A and A^T applications per image in the forward
    return {"op": "modl", "config": "c4", "batch": c.batch, "recompute": recompute,
            "forward_s": tf, "backward_s": tb, "backward_over_forward": tb / tf,
            "images_per_s_train": c.batch / (tf + tb), "projector_applications_forward": n_proj,
            "peak_mem_gb": torch.cuda.max_memory_allocated() / 1e9, "loss": float(loss.detach()),
            "projector_schedule": schedule, "cudnn_search": cudnn_search}


def c3(dev, iters=50, warmup=3, reps=20, streams=0, autotune=False, plain=False):
    """The 64 uneven scans (N 128..768, 90..720 views), `iters` ADMM-TV
    iterations each: one ct_admm_tv_solve_batch call against the same scans
    solved one after another with ct_admm_tv_solve (the reference's loop),
    both from device-resident data, CUDA events.  plain: also the per-scan
    loops without graphs and through the drop-in ADMM."""
    cfgs = workloads.batched_configs()
    n = len(cfgs)
    tune_s = 0.0
    if autotune:
        import time

        t0 = time.perf_counter()
        seen = set()
        for c in cfgs:
            if (c.n, c.n_views) not in seen:
                seen.add((c.n, c.n_views))
                linop.XRayTransform2D((c.n, c.n), c.angles, det_count=c.det_count).autotune(reps=5)
        tune_s = time.perf_counter() - t0
    ys, xs, wss, descs, its, keep = [], [], [], [], [], []
    for c in cfgs:
        A = linop.XRayTransform2D((c.n, c.n), c.angles, det_count=c.det_count)
        x_gt = torch.from_numpy(c.phantom()).to(dev)
        y = A(x_gt)
        y = y + c.noise * y.abs().max() * torch.randn(y.shape, generator=torch.Generator().manual_seed(c.noise_seed)).to(dev)
        g = A.geometry()
        d = _lib.AdmmTvDesc(g, iters, c.cg_maxiter, c.cg_tol, 0.0, c.lam, 0.0, c.rho, 0.5, 1.0, 1)
        nb = _lib.c_size_t()
        _lib.call("ct_admm_tv_workspace", ctypes.addressof(d), ctypes.addressof(nb))
        keep.append(A)
        ys.append(y)
        xs.append(torch.zeros((c.n, c.n), device=dev))
        wss.append(_device.workspace(nb.value))
        its.append(torch.zeros((iters, _lib.CT_ITSTAT_FIELDS), dtype=torch.float64, device=dev))
        descs.append(d)
    P = ctypes.c_void_p
    D = (_lib.AdmmTvDesc * n)(*descs)
    Y = (P * n)(*[t.data_ptr() for t in ys])
    X = (P * n)(*[t.data_ptr() for t in xs])
    I = (P * n)(*[t.data_ptr() for t in its])
    W = (P * n)(*[t.data_ptr() for t in wss])
    B = (_lib.c_size_t * n)(*[t.numel() for t in wss])
    s = torch.cuda.current_stream()

    def batched():
        for x in xs:
            x.zero_()
        _lib.call("ct_admm_tv_solve_batch", ctypes.addressof(D), n, ctypes.addressof(Y), ctypes.addressof(X),
                  ctypes.addressof(I), 0, ctypes.addressof(W), ctypes.addressof(B), streams, s.cuda_stream)

    def looped():
        for k in range(n):
            xs[k].zero_()
            _lib.call("ct_admm_tv_solve", ctypes.addressof(descs[k]), ys[k].data_ptr(), xs[k].data_ptr(),
                      its[k].data_ptr(), 0, wss[k].data_ptr(), wss[k].numel(), s.cuda_stream)

    tb, _ = _time(batched, s, warmup, reps)
    tl, _ = _time(looped, s, warmup, reps)
    inter = sum(c.n * c.n * c.n_views for c in cfgs)
    batched()
    torch.cuda.synchronize()
    cg = torch.stack([t[:, _lib.CT_ITSTAT_CG_ITERS] for t in its]).cpu()
    # projector work actually run: one forward/adjoint pair per CG step plus
    # the pair of each iteration's start (A x, A^T A x), skipped only when x
    # did not change
    pairs = sum(float(cg[k].sum() + iters) * cfgs[k].n ** 2 * cfgs[k].n_views for k in range(n))
    out = {"op": "c3", "scans": n, "iters": iters, "streams": streams, "batched_s": tb,
           "looped_s": tl, "speedup": tl / tb, "scans_per_s": n / tb, "interactions_per_application": inter,
           "mean_cg_iters": float(cg.mean()), "autotune_s": tune_s,
           "projection_pair_interactions": pairs}
    if plain:
        # the fused per-scan solver with every launch issued from the host
        for d in descs:
            d.use_graph = 0
        tn, _ = _time(looped, s, 1, max(1, reps // 2))
        for d in descs:
            d.use_graph = 1

        # the plain drop-in: scico's ADMM loop on the GPU operators, one scan
        # after another (CG convergence tested on the host every step)
        def generic():
            for k, c in enumerate(cfgs):
                f = loss.SquaredL2Loss(y=ys[k], A=keep[k])
                C = linop.FiniteDifference((c.n, c.n), append=0)
                ADMM(f=f, g_list=[c.lam * functional.L21Norm()], C_list=[C], rho_list=[c.rho], maxiter=iters,
                     subproblem_solver=LinearSubproblemSolver(cg_kwargs={"tol": c.cg_tol, "maxiter": c.cg_maxiter}),
                     fused=False).solve()

        tg, _ = _time(generic, s, 0, 1)
        out.update({"looped_plain_launch_s": tn, "speedup_vs_plain_launch": tn / tb,
                    "looped_generic_s": tg, "speedup_vs_generic": tg / tb})
    return out


if __name__ == "__main__":
    main()
