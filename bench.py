"""Benchmark: converged views/sec of the depth-to-view pipeline on one GB300 -- the headline metric, "views/sec to
energy gap <= 1e-4: learned + batched vs plain solver, same GB300".

Workload (default "c5", the full pipeline the metric is quoted on): one synthetic 9x9 light field of 1024x1024
RGB float32 views (rendered at 2048^2 and box-decimated 2x, 5 planes + 20 Gaussian depth bumps, baseline 0.03,
noise 0.005), its 80 inputs warped to 32 target cameras of 2048x2048 (2x super-resolution) and reconstructed with
the gradient-constraint formulation (IBR_gradient) solved by conjugate gradient with FP32 iterates and FP64 dot
products until the certified relative energy gap is <= 1e-4. One step = the 32 targets.

  value : views/sec of the learned + batched arm (BF16 view stacks, the encoder-decoder's warm start, all 32
          targets in one lfrv_render_views_warm_dev call) with inputs resident in HBM
  config.modes / speedup_vs_plain : every arm (plain FP32 one target at a time -- the plain solver --, plain
          batched, BF16 batched, learned + BF16 batched) on the same targets and the same GPU
  e2e   : the learned + batched arm through the host-buffer C ABI call (lfrv_render_views_warm), from pinned host
          memory, with the light field's upload and the 32 outputs' download inside the timed region
  roofline : the dominant kernel of the plain step (by device time), algorithmic bytes per launch / its average
          CUDA-event duration on the launch stream
  cpu_baseline : the FP32 CPU restatement of the reference path (oracle port, OpenMP over the host cores) on the
          centre target
  vs_fp64 : the centre target against the FP64 CPU oracle run on the GPU's warps

Other workloads (--workload): c1 (3x3 256^2, IBR_color 300 x 300 iterations), c2 (5x5 512^2 -> 1024^2, one target),
c3 (batched targets of uneven size), c4 (learned warm start trained in the run, 512^2), tv (the corrected
IBR_color to a certified gap of 1e-4 on the 3x3 256^2 scene), net (the network alone).

`--impl reference` times the CPU restatement alone as the reference arm (the reference's own path needs Qt, glm,
OpenGL and its CUDA runtime and cannot run here).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "light-field-remote-vision_gb300"))

WORKLOADS = {
    "c5": dict(preset=2, algorithm=1, steps=5, warmup=3,
               name="full pipeline: 9x9 LF of 1024^2 views (80 inputs rendered at 2048^2 and box-decimated, 5 planes + "
                    "20 bumps) -> 32 targets of 2048^2 (dsf 2), IBR_gradient + CG to gap 1e-4; learned warm start + BF16 "
                    "stacks + batched vs the plain FP32 solver one target at a time"),
    "c3": dict(preset=2, algorithm=1, steps=3, warmup=3,
               name="batched: 64 targets of 256^2..1024^2 from 8 seeded 9x9 light fields (baselines 0.01..0.05, dsf 1 "
                    "or 2); two targets per field without SR run the corrected IBR_color (TV_F to a certified gap of "
                    "1e-4), the others IBR_gradient + CG to gap 1e-4; one lfrv_render_views_dev call"),
    "c2": dict(preset=2, algorithm=1, steps=200, warmup=5,
               name="5x5 LF 512^2 -> 1024^2 (dsf 2), 24 views, IBR_gradient + CG to gap 1e-4"),
    "c1": dict(preset=1, algorithm=0, steps=10, warmup=3,
               name="3x3 LF 256^2, 8 views, IBR_color primal-dual TV, 300 x 300 iterations"),
    "c4": dict(preset=1, algorithm=1, steps=3, warmup=3,
               name="learned warm start as configured: trained on 4000 seeded 3x3 light fields of 512^2 (3 planes + 20 "
                    "bumps, generated on the GPU) against plain solutions at gap 1e-6; 256 held-out scenes, IBR_gradient "
                    "+ CG to gap 1e-4 from the network's seed, batched, vs the plain start"),
    "tv": dict(preset=1, algorithm=0, steps=10, warmup=3,
               name="3x3 LF 256^2, 8 views, IBR_color corrected mode: the weighted TV_F objective to a certified "
                    "relative primal-dual gap of 1e-4 (FISTA + FGP)"),
    "net": dict(preset=0, algorithm=-1, steps=10, warmup=3,
                name="learned warm start network alone: one 512^2 inference and one training step of 4"),
}


def make_config(lfrv, wl: str, sc):
    p = sc.params
    V = sc.views.shape[0]
    if wl == "c2":
        return lfrv.default_config(w=p.w, h=p.h, dsf=p.dsf, nviews=V, nchannels=3, sigma_sensor=0.005,
                                   ugrad_threshold=1.0, lambda_=0.05, lambda_max_factor=100.0, faithful=0,
                                   cg_gap_tol=1e-4, cg_max_iter=500, hole_fill_iter=500)
    if wl == "tv":
        return lfrv.default_config(w=p.w, h=p.h, dsf=p.dsf, nviews=V, nchannels=3, sigma_sensor=0.01,
                                   ugrad_threshold=1.0, lambda_=0.05, lambda_max_factor=100.0, niter=500, nmeta_iter=1,
                                   early_exit=0, faithful=0, cg_gap_tol=1e-4)
    return lfrv.default_config(w=p.w, h=p.h, dsf=p.dsf, nviews=V, nchannels=3, sigma_sensor=0.01,
                               ugrad_threshold=1.0, lambda_=0.05, lambda_max_factor=100.0, niter=300, nmeta_iter=1,
                               early_exit=0, faithful=1)


def algorithmic_bytes(kernel: str, V: int, n: int, N: int, ks: int, cg_iters: int = 0,
                      rof_iters: int = 0) -> float | None:
    """Compulsory DRAM bytes of one launch of `kernel` (FP32 = 4 B; V views of n pixels, N target pixels)."""
    table = {
        # per CG iteration the state vectors x, r, d are each read and written once: 72 B per pixel (q is not
        # materialised; the FP64 scalars are negligible)
        "cg_persistent": cg_iters * 72 * N,
        # inverse map (bucket starts + 4 B entries), per source pixel tau 8 B + colour 12 B + Sobel 8 B +
        # weight 4 B; vis 1 B, U 12 B, g_x, g_y, mask 12 B written per target pixel
        "gradient_setup": 4 * N + 4 * V * n + 32 * V * n + 25 * N,
        "zbuffer_splat": 12 * V * n + 8 * N,          # depth (z, dz/dx, dz/dy) read, 64-bit key per target pixel
        "tau": 12 * V * n + 4 * N + 16 * V * n,       # depth + target depth map read, tau and dp written
        "bucket_build": 8 * V * n * 2 + 4 * V * n + 8 * (N + 2 * N),
        "weights": 16 * V * n + 8 * N + 4 * V * n,    # tau + dp, gradient planes, weights written
        "vis_any": 4 * N + 8 * V * n + 4 * V * n + 1 * N,
        "initial_image": 24 * V * n + 4 * V * n + 4 * N + 16 * N,
        "hole_list": 1 * N,
        "hole_fill_iter": None,
        "sobel": 12 * V * n + 8 * V * n,
        "u_gradient": (8 + 4 + 8) * V * n + 4 * V * n + 4 * N + 12 * N,
        "cg_init": 12 * N + 8 * N + 24 * N,
        "cg_apply": 12 * N + 12 * N,
        "cg_update": 48 * N + 24 * N,
        "cg_dir": 24 * N + 12 * N,
        "cg_energy": 24 * N + 8 * N,
        "rof_iter": 88 * N,
        # all inner iterations of one ISTA step in one launch: 88 B per target pixel per iteration
        "rof_persistent": 88 * N * rof_iters,
        "residual": 12 * N + 24 * V * n + 12 * V * n,
        # the FGP iterations of one FISTA step in one launch; per iteration the FP64 dual p and momentum q (48 B
        # each), F (12), lam, 1/L, g (4 each) read and p, q written (96): 216 B per target pixel (FP32 and
        # double-float arithmetic of the dual both keep FP64 storage)
        "tv_fgp": 200 * 216 * N,
        "tv_fgp_df": 200 * 216 * N,
        "dataterm_F": 12 * V * n + 8 * V * n + 4 * V * n + 12 * N + 12 * N,
    }
    return table.get(kernel)


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from ncu --set full captures (summaries in
# profiles/): the C2 step (5x5 light field of 512^2 views -> the 1024^2 target), the C1 ROF launch (256^2), and
# for the C5 target (80 views of 1024^2 -> 2048^2) the z-buffer splat's C2 capture scaled by its algorithmic
# bytes (at C2 its traffic is 1.03 x its algorithmic bytes: depth maps read once, keys in L2).
NCU_TRAFFIC_BYTES = {
    ("zbuffer_splat", 1024 * 1024): 83.942912e6 + 2.418432e6 + 0.335616e6,
    ("gradient_setup", 1024 * 1024): 223.959296e6 + 18.378240e6,
    ("cg_persistent", 1024 * 1024): 21.045248e6 + 0.000512e6,
    ("zbuffer_splat", 2048 * 2048): 1.03 * (12 * 80 * 1024 * 1024 + 8 * 2048 * 2048),
    ("rof_persistent", 256 * 256): 3.427584e6 + 0.028928e6,
}


def barrier() -> None:
    """All ranks meet here before a timed region; nothing to do in a single process."""
    import torch

    if torch.distributed.is_available() and torch.distributed.is_initialized():
        torch.distributed.barrier()


def max_over_ranks(x: float, device: str = "cuda") -> float:
    """The largest x over the ranks (the slowest replica's time); x itself in a single process."""
    import torch

    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def sample_clocks(path: str):
    return subprocess.Popen(
        ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
         "--format=csv,noheader,nounits", "-lms", "50", "-i", os.environ.get("LOCAL_RANK", "0")],
        stdout=open(path, "w"), stderr=subprocess.DEVNULL)


def summarize_clocks(path: str) -> dict:
    sm, mx, reasons = [], [], set()
    try:
        for line in open(path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for name, val in zip(names, f[5:9]):
                if val.lower() in ("active", "1", "yes"):
                    reasons.add(name)
    except OSError:
        pass
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
            "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm() -> tuple[float, str]:
    try:
        d = json.load(open(ROOT / "MEASURED_PEAKS.json"))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_step(pyoracle, wl: str, cfg, sc, algorithm: int) -> float:
    t0 = time.perf_counter()
    tau, dpart, _ = pyoracle.warp(sc.depth, sc.cams, sc.target)
    if algorithm == 1:
        pyoracle.ibr_gradient(cfg, sc.views, tau, dpart, prec=1)
    else:
        pyoracle.ibr_color(cfg, sc.views, tau, dpart, prec=1)
    return time.perf_counter() - t0


def run_reference(args, rank: int) -> None:
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    import lfrv
    import pyoracle

    wl = WORKLOADS[args.workload]
    if args.workload == "net":
        print(json.dumps({"impl": "reference", "unavailable": "the learned network has no reference counterpart"}))
        return
    if args.workload == "c5":
        p, sc, targets, _ = c5_scene(lfrv)
        sc.target = targets[0]
        cfg = c5_config(lfrv, p, sc.views.shape[0])
        sample = "the centre target of the 32 per step"
        metric = "views/sec to energy gap <=1e-4 (learned+batched vs plain solver, same GB300)"
    else:
        sc = lfrv.synth_scene(lfrv.scene_params(wl["preset"]))
        cfg = make_config(lfrv, args.workload, sc)
        sample = "one full view per step"
        metric = "views/sec to energy gap <=1e-4"
    if args.workload == "c1":
        cfg.niter = 30  # bounded sample: 30 x 30 iterations; the value is scaled to the 300 x 300 step below
    algorithm = max(0, wl["algorithm"])
    # Bounded sample: one warm-up view at most, then full views until K views or a ~150 s budget (warm-up included)
    # is used; at least one view is timed.
    t_start = time.perf_counter()
    if args.warmup > 0:
        cpu_step(pyoracle, args.workload, cfg, sc, algorithm)
    times = []
    while len(times) < args.steps and (not times or time.perf_counter() - t_start + times[-1] < 150.0):
        times.append(cpu_step(pyoracle, args.workload, cfg, sc, algorithm))
    sec = sum(times) / len(times)
    if args.workload == "c1":
        sec *= 100.0  # ROF work scales with niter^2
    cores = os.cpu_count()
    v = 1.0 / sec
    line = {"impl": "reference", "metric": metric, "value": v, "unit": "views/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": wl["name"]},
            "cpu_baseline": {"value": v, "unit": "views/s", "cores": cores, "kind": "port",
                             "sample": f"{len(times)} full views (warp + solve; {sample}) timed of {args.steps} "
                                       f"requested (150 s budget), FP32 CPU restatement, OpenMP"},
            "e2e": {"value": v, "unit": "views/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_net(args, rank: int, world: int) -> None:
    """The learned warm start network alone: one 512^2 inference and one training step of 4 images, random inputs
    of the network's shape, CUDA events on the library's stream after warm-up."""
    import torch
    import lfrv

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream()
    ctx = lfrv.Context(dev, stream.cuda_stream)
    net = lfrv.WarmStart(ctx, seed=1)
    H = W = 512
    B = 4
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand((B, H, W, lfrv.WARMSTART_CHANNELS), device="cuda", generator=g).to(torch.bfloat16)
    u0 = torch.rand((B, 3, H, W), device="cuda", generator=g)
    tg = u0 + 0.01 * torch.randn((B, 3, H, W), device="cuda", generator=g)
    pred = torch.zeros_like(u0)
    torch.cuda.synchronize()

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    l0 = ctx.launch_count()
    fwd_ms = timed(lambda: net.forward_dev(1, H, W, x[0].data_ptr(), u0[0].data_ptr(), pred[0].data_ptr()))
    launches = ctx.launch_count() - l0
    train_ms = timed(lambda: net.train_step_dev(B, H, W, x.data_ptr(), u0.data_ptr(), tg.data_ptr(), 1e-4))
    gflop = 34.6  # 2 M N K of the 12 convolutions and the head at 512^2 (unpadded K)
    if rank == 0:
        print(json.dumps({"metric": "learned warm start inference images/sec", "value": 1e3 / fwd_ms,
                          "unit": "images/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": fwd_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "bf16 (fp32 accumulation)", "data": "random inputs of the network's shape",
                          "config": {"workload": WORKLOADS["net"]["name"], "forward_ms": fwd_ms,
                                     "train_step_ms_batch4": train_ms, "forward_tflops": gflop / fwd_ms,
                                     "forward_launches": launches // max(1, args.warmup + args.steps)}}),
              flush=True)
    net.close()
    ctx.close()


def batch_scenes(lfrv):
    """C3's inputs: 8 seeded 9x9 light fields (planes + bumps) of uneven size (target side drawn uniformly from
    256, 384, 512, 768, 1024; SR factor 1 or 2 where the views stay at least 256 wide; baseline drawn from
    0.01..0.05), 8 target cameras each (the centre camera shifted by fractions of the baseline)."""
    import copy
    rng = np.random.default_rng(7)
    targets = [256, 384, 512, 768, 1024]
    fields = []
    for i in range(8):
        T = int(targets[rng.integers(0, len(targets))])
        dsf = int(rng.integers(1, 3)) if T >= 512 else 1
        p = lfrv.scene_params(2, w=T // dsf, h=T // dsf, grid=9, dsf=dsf, ss=dsf, seed=100 + i,
                              baseline=float(rng.uniform(0.01, 0.05)))
        sc = lfrv.synth_scene(p)
        tgts = []
        for k in range(8):
            t = copy.copy(sc.target)
            t.t[0] = sc.target.t[0] + ((k % 4) - 1.5) * 0.25 * p.baseline
            t.t[1] = sc.target.t[1] + ((k // 4) - 0.5) * 0.5 * p.baseline
            tgts.append(t)
        fields.append((sc, tgts))
    return fields


def run_batch(args, rank: int, world: int) -> None:
    """C3: one lfrv_render_views_dev call over 64 targets: two of the eight targets of each field without
    super-resolution run the corrected IBR_color (the TV_F objective to a certified gap of 1e-4; with SR factor 2
    it needs 150 to 200+ outer steps at these sizes), the others IBR_gradient with the corrected CG; against the
    same 64 targets rendered one lfrv_render_view_dev call at a time."""
    import torch
    import lfrv

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    wl = WORKLOADS[args.workload]
    t_gen = time.time()
    fields = batch_scenes(lfrv)
    t_gen = time.time() - t_gen
    stream = torch.cuda.Stream()
    ctx = lfrv.Context(dev, stream.cuda_stream)
    jobs, keep = [], []
    for sc, tgts in fields:
        cfg_cg = make_config(lfrv, "c2", sc)
        cfg_tv = make_config(lfrv, "tv", sc)
        cfg_tv.niter = 200  # outer-step cap of the TV jobs
        dv = torch.from_numpy(sc.views).cuda()
        dd = torch.from_numpy(sc.depth).cuda()
        keep += [dv, dd, cfg_cg, cfg_tv]
        for k, t in enumerate(tgts):
            out = torch.empty((3, t.height, t.width), device="cuda")
            keep.append(out)
            tv = k % 4 == 3 and sc.params.dsf == 1  # TV on the fields without super-resolution
            jobs.append(dict(cfg=cfg_tv if tv else cfg_cg, algorithm=0 if tv else 1, d_views=dv.data_ptr(),
                             d_depth=dd.data_ptr(), cams=sc.cams, target=t, d_out=out.data_ptr()))
    torch.cuda.synchronize()

    def batched():
        return ctx.render_views_dev(jobs)

    def one_by_one():
        return [ctx.render_view_dev(j["cfg"], j["algorithm"], j["d_views"], j["d_depth"], j["cams"], j["target"],
                                    j["d_out"]) for j in jobs]

    for _ in range(max(args.warmup, 3)):
        st = batched()
    one_by_one()
    torch.cuda.synchronize()
    clk_path = tempfile.mktemp(prefix="lfrv_clocks_")
    clk = sample_clocks(clk_path)
    l0 = ctx.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        st = batched()
    e1.record(stream)
    torch.cuda.synchronize()
    launches = ctx.launch_count() - l0
    sec = e0.elapsed_time(e1) / 1e3
    clk.terminate()
    clk.wait()
    clocks = summarize_clocks(clk_path)
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for _ in range(args.steps):
        st1 = one_by_one()
    s1.record(stream)
    torch.cuda.synchronize()
    sec_single = s0.elapsed_time(s1) / 1e3
    nv = len(jobs) * args.steps
    sizes = sorted({(j["target"].width) for j in jobs})
    tv = [i for i, j in enumerate(jobs) if j["algorithm"] == 0]
    cg = [i for i, j in enumerate(jobs) if j["algorithm"] == 1]
    if rank == 0:
        line = {"metric": "views/sec to energy gap <=1e-4", "value": world * nv / sec, "unit": "views/s",
                "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
                "ms_per_step": sec * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32 (TV dual: FP64 storage, FP32 / double-float arithmetic)",
                "data": "synthetic (seeded planes + bumps light fields)",
                "config": {"workload": wl["name"], "targets_per_step": len(jobs), "target_sizes": sizes,
                           "tv_targets": len(tv), "cg_targets": len(cg),
                           "scene_generation_seconds": round(t_gen, 1),
                           "cg_iterations": [st[i].outer_iterations for i in cg][:8],
                           "tv_outer_steps": [st[i].outer_iterations for i in tv][:8],
                           "max_gap": max(s.gap for s in st),
                           "same_iterations_as_one_at_a_time": all(a.outer_iterations == b.outer_iterations
                                                                   for a, b in zip(st, st1)),
                           "one_at_a_time_views_per_s": nv / sec_single,
                           "batching_gain": sec_single / sec,
                           "l2": "the 64 targets' buffers exceed L2 (no flush needed)"},
                "clocks": clocks, "gpu_launches": launches, "roofline": None, "cpu_baseline": None,
                "e2e": None}  # device-pointer batch API only: no host-buffer leg for this workload
        print(json.dumps(line), flush=True)
    ctx.close()


def run_warm(args, rank: int, world: int) -> None:
    """Learned warm start (c4) as configured: 4000 seeded 3x3 light fields of 512^2 (planes 1.0 / 1.5 / 2.5 plus 20
    Gaussian depth bumps), generated on the GPU, train the network (untimed) on their centre targets, streamed in
    chunks of 100 (network input, anchor, and the plain solution converged to gap 1e-6); then 256 held-out scenes:
    iterations and views/sec to gap 1e-4 from the plain start (the anchor) and from the network's prediction, one
    target at a time and batched."""
    import torch
    import lfrv

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    wl = WORKLOADS[args.workload]
    W = 512
    n_train, n_test, chunk = 4000, 256, 100
    ctx = lfrv.Context(dev)

    def params(seed):
        return lfrv.scene_params(1, w=W, h=W, seed=int(seed), nbumps=20, bump_amp=0.1, bump_sigma_px=30.0)

    V = 8

    def generate(seed, views, depth):
        cams, target = ctx.synth_scene_dev(params(seed), views.data_ptr(), depth.data_ptr())
        return cams, target

    def cfg_of(tol):
        p = params(0)
        return lfrv.default_config(w=p.w, h=p.h, dsf=p.dsf, nviews=V, nchannels=3, sigma_sensor=0.005, lambda_=0.05,
                                   faithful=0, cg_gap_tol=tol, cg_max_iter=500, hole_fill_iter=500)

    cfg6, cfg4 = cfg_of(1e-6), cfg_of(1e-4)
    net = lfrv.WarmStart(ctx, seed=1)
    g = torch.Generator().manual_seed(0)
    steps_per_chunk, bs = 40, 4
    views = torch.zeros((V, 3, W, W), device="cuda")
    depth = torch.zeros_like(views)
    X = torch.zeros((chunk, W, W, 48), dtype=torch.bfloat16, device="cuda")
    U0 = torch.zeros((chunk, 3, W, W), device="cuda")
    S = torch.zeros((chunk, 3, W, W), device="cuda")
    t_gen = t_feat = t_train = 0.0
    losses = []
    for c0 in range(0, n_train, chunk):
        for i in range(chunk):
            t0 = time.time()
            cams, target = generate(1000 + c0 + i, views, depth)
            t_gen += time.time() - t0
            t0 = time.time()
            ctx.warmstart_features_dev(cfg6, views.data_ptr(), depth.data_ptr(), cams, target, X[i].data_ptr(),
                                       U0[i].data_ptr(), S[i].data_ptr())
            torch.cuda.synchronize()
            t_feat += time.time() - t0
        t0 = time.time()
        for _ in range(steps_per_chunk):
            idx = torch.randperm(chunk, generator=g)[:bs].cuda()
            xb, ub, sb = X[idx].contiguous(), U0[idx].contiguous(), S[idx].contiguous()
            torch.cuda.synchronize()
            losses.append(net.train_step_dev(bs, W, W, xb.data_ptr(), ub.data_ptr(), sb.data_ptr(), 5e-4))
        torch.cuda.synchronize()
        t_train += time.time() - t0
    # held-out scenes: prediction quality on the first 32, then the timed arms over all 256
    mse_plain = mse_warm = 0.0
    pi = torch.zeros((3, W, W), device="cuda")
    for i in range(32):
        cams, target = generate(100000 + i, views, depth)
        ctx.warmstart_features_dev(cfg6, views.data_ptr(), depth.data_ptr(), cams, target, X[0].data_ptr(),
                                   U0[0].data_ptr(), S[0].data_ptr())
        net.forward_dev(1, W, W, X[0].data_ptr(), U0[0].data_ptr(), pi.data_ptr())
        torch.cuda.synchronize()
        mse_plain += float(((U0[0] - S[0]) ** 2).mean()) / 32
        mse_warm += float(((pi - S[0]) ** 2).mean()) / 32
    del X, U0, S, views, depth
    test_views = torch.zeros((n_test, V, 3, W, W), device="cuda")
    test_depth = torch.zeros_like(test_views)
    outs = torch.empty((n_test, 3, W, W), device="cuda")
    jobs = []
    for i in range(n_test):
        cams, target = generate(100000 + i, test_views[i], test_depth[i])
        jobs.append(dict(cfg=cfg4, algorithm=1, d_views=test_views[i].data_ptr(), d_depth=test_depth[i].data_ptr(),
                         cams=cams, target=target, d_out=outs[i].data_ptr()))
    torch.cuda.synchronize()

    def plain_single():
        return [ctx.render_view_dev(j["cfg"], 1, j["d_views"], j["d_depth"], j["cams"], j["target"], j["d_out"])
                for j in jobs]

    def warm_single():
        return [net.render_view_dev(j["cfg"], j["d_views"], j["d_depth"], j["cams"], j["target"], j["d_out"])
                for j in jobs]

    def plain_batched():
        return ctx.render_views_dev(jobs)

    def warm_batched():
        return ctx.render_views_dev(jobs, net)

    results = {}
    clocks, launches = None, None
    for name, fn in (("plain_single", plain_single), ("warm_single", warm_single), ("plain_batched", plain_batched),
                     ("warm_batched", warm_batched)):
        for _ in range(max(args.warmup, 3)):
            st = fn()
        torch.cuda.synchronize()
        if name == "warm_batched":
            clk_path = tempfile.mktemp(prefix="lfrv_clocks_")
            clk = sample_clocks(clk_path)
            l0 = ctx.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            st = fn()
        e1.record()
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1e3
        if name == "warm_batched":
            launches = ctx.launch_count() - l0
            clk.terminate()
            clk.wait()
            clocks = summarize_clocks(clk_path)
        its = [s.outer_iterations for s in st]
        results[name] = dict(views_per_s=len(jobs) * args.steps / sec, ms_per_target=1e3 * sec / (len(jobs) * args.steps),
                             cg_iterations_mean=float(np.mean(its)), cg_iterations_total=int(sum(its)),
                             max_gap=float(max(s.gap for s in st)))
    if rank == 0:
        wb = results["warm_batched"]
        line = {"metric": "views/sec to energy gap <=1e-4", "value": world * wb["views_per_s"], "unit": "views/s",
                "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
                "ms_per_step": 1e3 * len(jobs) / wb["views_per_s"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32 iterates, bf16 network",
                "data": "synthetic (seeded planes + bumps light fields, generated on the GPU)",
                "config": {"workload": wl["name"], "targets_per_step": len(jobs), "target": [W, W],
                           "train_scenes": n_train, "train_steps": len(losses), "train_batch": bs,
                           "train_seconds": round(t_train, 2), "features_seconds": round(t_feat, 2),
                           "scene_generation_seconds": round(t_gen, 2),
                           "train_loss_first_last": [losses[0], float(np.mean(losses[-20:]))],
                           "heldout_scenes": n_test, "heldout_mse_plain_start": mse_plain,
                           "heldout_mse_warm_start": mse_warm, "modes": results,
                           "learned_batched_vs_plain_single": wb["views_per_s"] / results["plain_single"]["views_per_s"],
                           "l2": "256 targets of 512^2 with 8 views each exceed L2 (no flush needed)"},
                "clocks": clocks, "gpu_launches": launches, "roofline": None, "cpu_baseline": None}
        print(json.dumps(line), flush=True)
    net.close()
    ctx.close()


def c5_scene(lfrv):
    """The c5 light field and its 32 target cameras (the rendered centre camera first, then 31 shifted by fractions
    of the baseline), plus 4 other cameras whose features train the network."""
    import copy

    p = lfrv.scene_params(2, w=1024, h=1024, grid=9, dsf=2, ss=2, seed=7000)
    sc = lfrv.synth_scene(p)

    def shifted(i, n_side, scale):
        t = copy.copy(sc.target)
        t.t[0] = sc.target.t[0] + ((i % n_side) - (n_side - 1) / 2) * scale * p.baseline
        t.t[1] = sc.target.t[1] + ((i // n_side) - (n_side - 1) / 2) * scale * p.baseline
        return t

    targets = [copy.copy(sc.target)] + [shifted(i, 6, 0.08) for i in range(31)]
    train_targets = [shifted(i, 2, 0.37) for i in range(4)]
    return p, sc, targets, train_targets


def c5_config(lfrv, p, V, tol=1e-4, bf16=False):
    return lfrv.default_config(w=p.w, h=p.h, dsf=p.dsf, nviews=V, nchannels=3, sigma_sensor=0.005, lambda_=0.05,
                               faithful=0, cg_gap_tol=tol, cg_max_iter=500, hole_fill_iter=500,
                               bf16_storage=1 if bf16 else 0)


def run_full(args, rank: int, world: int) -> None:
    """Full pipeline (c5), BASELINE's metric: one 9x9 light field, 32 target cameras, every arm timed over the 32
    targets on the same GPU: plain FP32 one at a time (the plain solver), plain FP32 batched, BF16 stacks batched,
    and learned + batched (BF16 stacks, warm start, one batched call) -- the headline value. The network is trained
    in the run on 512^2 crops of 4 other targets' 2048^2 features (untimed)."""
    import torch
    import lfrv

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    wl = WORKLOADS["c5"]
    t_gen = time.time()
    p, sc, targets, train_targets = c5_scene(lfrv)
    t_gen = time.time() - t_gen
    V = sc.views.shape[0]
    H, W = sc.gt.shape[1], sc.gt.shape[2]
    stream = torch.cuda.Stream()
    ctx = lfrv.Context(dev, stream.cuda_stream)
    cfg32, cfg16 = c5_config(lfrv, p, V), c5_config(lfrv, p, V, bf16=True)
    views = torch.from_numpy(sc.views).cuda()
    views_bf16 = views.to(torch.bfloat16)
    depth = torch.from_numpy(sc.depth).cuda()
    torch.cuda.synchronize()
    # training data for the network: features of 4 targets at 2048^2, random 512^2 crops
    t_feat = time.time()
    X = torch.zeros((len(train_targets), H, W, 48), dtype=torch.bfloat16, device="cuda")
    U0 = torch.zeros((len(train_targets), 3, H, W), device="cuda")
    S = torch.zeros((len(train_targets), 3, H, W), device="cuda")
    torch.cuda.synchronize()
    for i, t in enumerate(train_targets):
        ctx.warmstart_features_dev(c5_config(lfrv, p, V, tol=1e-6, bf16=True), views_bf16.data_ptr(), depth.data_ptr(),
                                   sc.cams, t, X[i].data_ptr(), U0[i].data_ptr(), S[i].data_ptr())
    torch.cuda.synchronize()
    t_feat = time.time() - t_feat
    net = lfrv.WarmStart(ctx, seed=1)
    rng = np.random.default_rng(0)
    steps, bs, crop = 1000, 4, 512
    t_train = time.time()
    for _ in range(steps):
        ii = rng.integers(0, len(train_targets), bs)
        ys = rng.integers(0, (H - crop) // 8 + 1, bs) * 8
        xs = rng.integers(0, (W - crop) // 8 + 1, bs) * 8
        xb = torch.stack([X[i, y:y + crop, x:x + crop] for i, y, x in zip(ii, ys, xs)]).contiguous()
        ub = torch.stack([U0[i, :, y:y + crop, x:x + crop] for i, y, x in zip(ii, ys, xs)]).contiguous()
        sb = torch.stack([S[i, :, y:y + crop, x:x + crop] for i, y, x in zip(ii, ys, xs)]).contiguous()
        torch.cuda.synchronize()
        net.train_step_dev(bs, crop, crop, xb.data_ptr(), ub.data_ptr(), sb.data_ptr(), 5e-4)
    torch.cuda.synchronize()
    t_train = time.time() - t_train
    del X, U0, S
    outs = {k: [torch.empty((3, H, W), device="cuda") for _ in targets]
            for k in ("plain_single", "plain_batched", "bf16_batched", "learned_batched")}

    def jobs(name, cfg, vp):
        return [dict(cfg=cfg, algorithm=1, d_views=vp, d_depth=depth.data_ptr(), cams=sc.cams, target=t,
                     d_out=outs[name][i].data_ptr()) for i, t in enumerate(targets)]

    j_ps = jobs("plain_single", cfg32, views.data_ptr())
    j_pb = jobs("plain_batched", cfg32, views.data_ptr())
    j_bb = jobs("bf16_batched", cfg16, views_bf16.data_ptr())
    j_wb = jobs("learned_batched", cfg16, views_bf16.data_ptr())
    arms = (("plain_single", lambda: [ctx.render_view_dev(j["cfg"], 1, j["d_views"], j["d_depth"], j["cams"],
                                                          j["target"], j["d_out"]) for j in j_ps]),
            ("plain_batched", lambda: ctx.render_views_dev(j_pb)),
            ("bf16_batched", lambda: ctx.render_views_dev(j_bb)),
            ("learned_batched", lambda: ctx.render_views_dev(j_wb, net)))
    results = {}
    clocks, launches = None, None
    torch.cuda.synchronize()
    for name, fn in arms:
        for _ in range(args.warmup):
            st = fn()
        torch.cuda.synchronize()
        barrier()
        headline = name == "learned_batched"
        if headline:
            clk_path = tempfile.mktemp(prefix="lfrv_clocks_")
            clk = sample_clocks(clk_path)
            l0 = ctx.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            st = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        sec = max_over_ranks(e0.elapsed_time(e1) / 1e3)  # the slowest replica's time
        if headline:
            launches = ctx.launch_count() - l0
            clk.terminate()
            clk.wait()
            clocks = summarize_clocks(clk_path)
        results[name] = dict(views_per_s=len(targets) * args.steps / sec,
                             cg_iterations=int(sum(s.outer_iterations for s in st)),
                             max_gap=float(max(s.gap for s in st)))
    # every arm against the plain FP32 solver's outputs (same targets)
    ref = [o.cpu().numpy() for o in outs["plain_single"]]
    for name in ("plain_batched", "bf16_batched", "learned_batched"):
        got = [o.cpu().numpy() for o in outs[name]]
        results[name]["max_abs_vs_plain_fp32"] = float(max(np.abs(a - b).max() for a, b in zip(got, ref)))
        results[name]["psnr_vs_plain_fp32_min_db"] = float(min(lfrv.psnr(a, b) for a, b in zip(got, ref)))
    centre = {name: outs[name][0].cpu().numpy() for name in outs}
    psnr_gt = {name: lfrv.psnr(centre[name], sc.gt) for name in outs}

    # the dominant kernel of the plain step: per-kernel device time over one pass of the 32 targets
    ctx.profile_enable(True)
    st_prof = [ctx.render_view_dev(j["cfg"], 1, j["d_views"], j["d_depth"], j["cams"], j["target"], j["d_out"])
               for j in j_ps]
    prof = ctx.profile()
    ctx.profile_enable(False)
    n, N = p.w * p.h, H * W
    roof, kernels_ms = roofline_of(prof, V, n, N, p.dsf + 1, st_prof, None, len(targets))

    # end to end: the learned + batched arm from pinned host buffers through lfrv_render_views_warm
    hv = views_bf16.cpu().pin_memory()
    hd = torch.from_numpy(sc.depth).pin_memory()
    hos = [torch.empty((3, H, W), dtype=torch.float32).pin_memory() for _ in targets]
    hjobs = [dict(cfg=cfg16, algorithm=1, d_views=hv.data_ptr(), d_depth=hd.data_ptr(), cams=sc.cams, target=t,
                  d_out=o.data_ptr()) for t, o in zip(targets, hos)]
    for _ in range(max(1, args.warmup // 2)):
        ctx.render_views(hjobs, net)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.render_views(hjobs, net)
    # the call returns after its outputs are in host memory; the slowest replica's time
    e2e_sec = max_over_ranks(time.perf_counter() - t0)
    e2e = {"value": world * len(targets) * args.steps / e2e_sec, "unit": "views/s",
           "h2d_bytes_per_step": int(hv.numel() * 2 + hd.numel() * 4),
           "d2h_bytes_per_step": int(len(targets) * 3 * H * W * 4)}
    e2e_match = bool(all(np.array_equal(o.numpy(), w.cpu().numpy()) for o, w in zip(hos, outs["learned_batched"])))
    del hos

    # CPU legs on the centre target: the FP32 port timed (cpu_baseline), the FP64 oracle on the GPU's warps
    cpu, vs64 = None, None
    if rank == 0 and world == 1 and not args.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import pyoracle

        tau_g, dpart_g, _ = ctx.warp(sc.depth, sc.cams, targets[0])
        t0 = time.perf_counter()
        tau_c, dpart_c, _ = pyoracle.warp(sc.depth, sc.cams, targets[0])
        pyoracle.ibr_gradient(cfg32, sc.views, tau_c, dpart_c, prec=1)
        t_cpu = time.perf_counter() - t0
        del tau_c, dpart_c
        cpu = {"value": 1.0 / t_cpu, "unit": "views/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "the centre target of the 32 (warp of 80 views + IBR_gradient to gap 1e-4), FP32 CPU "
                         "restatement of the reference path, OpenMP"}
        ref64, rst64 = pyoracle.ibr_gradient(cfg32, sc.views, tau_g, dpart_g, prec=0)
        vs64 = {"target": "centre (rendered ground truth available)", "warps": "the GPU's (lfrv_warp_dev)",
                "plain_fp32_max_rel_err": rel_err(centre["plain_single"], ref64),
                "plain_fp32_cg_iterations": st_prof[0].outer_iterations, "fp64_cg_iterations": rst64.outer_iterations,
                "learned_batched_max_abs_err": float(np.abs(centre["learned_batched"] - ref64).max()),
                "psnr_to_render_fp64_db": lfrv.psnr(ref64, sc.gt),
                "psnr_to_render_learned_batched_db": psnr_gt["learned_batched"],
                "psnr_delta_learned_batched_db": psnr_gt["learned_batched"] - lfrv.psnr(ref64, sc.gt),
                "psnr_to_render_plain_fp32_db": psnr_gt["plain_single"]}
    if rank == 0:
        wb = results["learned_batched"]
        plain = results["plain_single"]["views_per_s"]
        line = {"metric": "views/sec to energy gap <=1e-4 (learned+batched vs plain solver, same GB300)",
                "value": world * wb["views_per_s"], "unit": "views/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * len(targets) / wb["views_per_s"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "bf16 stacks, f32 iterates, f64 dots", "data": "synthetic (seeded planes + bumps light field)",
                "config": {"workload": wl["name"], "views": V, "input": [p.h, p.w], "target": [H, W],
                           "targets_per_step": len(targets), "scene_generation_seconds": round(t_gen, 1),
                           "features_seconds": round(t_feat, 2), "train_seconds": round(t_train, 2),
                           "train": f"{steps} Adam steps of {bs} random {crop}^2 crops of 4 other targets' features",
                           "plain_views_per_s": plain, "speedup_vs_plain": wb["views_per_s"] / plain,
                           "modes": results, "psnr_to_render_centre_target": psnr_gt,
                           "e2e_outputs_equal_device_call": e2e_match,
                           "l2": "32 targets of 2048^2 from 80 views of 1024^2 exceed L2 (no flush needed)"},
                "vs_fp64": vs64, "clocks": clocks, "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu,
                "e2e": e2e, "kernels_ms_per_step": kernels_ms}
        print(json.dumps(line), flush=True)
    net.close()
    ctx.close()


def rel_err(a, b, floor: float = 1e-2) -> float:
    """Max over pixels of |a - b| / max(|b|, floor)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


def roofline_of(prof: dict, V: int, n: int, N: int, ks: int, stats, rof_iters, targets: int):
    """roofline of the dominant kernel in a per-kernel profile (launcher name -> (total ms, launches)) and the
    per-step milliseconds of every kernel."""
    dom = max(prof, key=lambda k: prof[k][0])
    dom_ms, dom_n = prof[dom]
    avg_s = dom_ms / 1e3 / dom_n
    cg_iters = float(np.mean([s.outer_iterations for s in stats])) if stats else 0
    abytes = algorithmic_bytes(dom, V, n, N, ks, cg_iters=cg_iters, rof_iters=rof_iters or 0)
    peak, peak_kind = measured_peak_hbm()
    roof = None
    if abytes:
        ach = abytes / avg_s / 1e9
        roof = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                "peak_source": peak_kind, "traffic": NCU_TRAFFIC_BYTES.get((dom, N)),
                "avg_launch_us": avg_s * 1e6, "algorithmic_bytes_per_launch": abytes}
        if roof["traffic"]:
            roof["dram_frac"] = roof["traffic"] / avg_s / 1e9 / peak
        # what bounds the kernel instead of HBM, from its ncu capture
        roof["limiter"] = {
            "cg_persistent": "two grid barriers per iteration and the FP64 block sums before them; r and d stay in "
                             "shared memory, so DRAM moves only the one-time read of g and u",
            "zbuffer_splat": "instruction issue (75% issue active): per source pixel four projected corners, a "
                             "two-triangle set-up and the coverage and depth of its pixel centres; DRAM traffic is "
                             "the algorithmic bytes",
            "gradient_setup": "latency of dependent gathers at 24% occupancy (63 register partials per lane)",
            "rof_persistent": "block barriers between the dual and primal phases and the grid barrier per super-step; "
                              "the working set is L2-resident",
        }.get(dom)
    kernels_ms = {k: v[0] / targets for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}
    return roof, kernels_ms


def run_ours(args, rank: int, world: int) -> None:
    import torch
    import lfrv

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    wl = WORKLOADS[args.workload]
    sc = lfrv.synth_scene(lfrv.scene_params(wl["preset"]))
    cfg = make_config(lfrv, args.workload, sc)
    V, _, h, w = sc.views.shape
    H, W = h * sc.params.dsf, w * sc.params.dsf
    n, N, ks = h * w, H * W, sc.params.dsf + 1
    stream = torch.cuda.Stream()
    views = torch.from_numpy(sc.views).cuda()
    depth = torch.from_numpy(sc.depth).cuda()
    out = torch.empty((3, H, W), device="cuda", dtype=torch.float32)
    ctx = lfrv.Context(dev, stream.cuda_stream)
    torch.cuda.synchronize()

    def step():
        return ctx.render_view_dev(cfg, wl["algorithm"], views.data_ptr(), depth.data_ptr(), sc.cams, sc.target,
                                   out.data_ptr())

    for _ in range(max(args.warmup, 3)):
        st = step()
    torch.cuda.synchronize()
    # the working set (24 views x 6 planes x 1 MB + the 1024^2 target state) exceeds nothing in L2 between
    # steps: each step rewrites > 300 MB of buffers, so consecutive steps start from a cold L2
    barrier()
    clk_path = tempfile.mktemp(prefix="lfrv_clocks_")
    clk = sample_clocks(clk_path)
    l0 = ctx.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    stats = [step() for _ in range(args.steps)]
    e1.record(stream)
    torch.cuda.synchronize()
    launches = ctx.launch_count() - l0
    ms = e0.elapsed_time(e1)
    clk.terminate()
    clk.wait()
    clocks = summarize_clocks(clk_path)
    sec = max_over_ranks(ms / 1e3)  # the slowest replica's time
    value = world * args.steps / sec

    # per-kernel device time over a second pass of the same steps (events on the launch stream)
    ctx.profile_enable(True)
    for _ in range(args.steps):
        step()
    prof = ctx.profile()
    ctx.profile_enable(False)
    roof, kernels_ms = roofline_of(prof, V, n, N, ks, [st], int(cfg.niter), args.steps)

    # end to end through the host-buffer C ABI call, pinned host memory
    hv = torch.from_numpy(sc.views).pin_memory()
    hd = torch.from_numpy(sc.depth).pin_memory()
    ho = torch.empty((3, H, W), dtype=torch.float32).pin_memory()
    for _ in range(2):
        ctx.render_view(cfg, wl["algorithm"], hv.data_ptr(), hd.data_ptr(), sc.cams, sc.target, ho.data_ptr())
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        ctx.render_view(cfg, wl["algorithm"], hv.data_ptr(), hd.data_ptr(), sc.cams, sc.target, ho.data_ptr())
    f1.record(stream)
    torch.cuda.synchronize()
    e2e_sec = max(f0.elapsed_time(f1) / 1e3, 1e-9)
    wall = time.perf_counter() - t0
    e2e_value = world * args.steps / max_over_ranks(max(e2e_sec, wall))  # the slowest replica's time

    cpu, vs64 = None, None
    if rank == 0 and world == 1 and not args.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import pyoracle

        ccfg = make_config(lfrv, args.workload, sc)
        if args.workload == "c1":
            ccfg.niter = 30
        t = cpu_step(pyoracle, args.workload, ccfg, sc, wl["algorithm"])
        if args.workload == "c1":
            t *= 100.0
        cpu = {"value": 1.0 / t, "unit": "views/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "one full view (warp + solve) of the same workload, FP32 CPU restatement, OpenMP"
                         + (" (30 x 30 of the 300 x 300 iterations, time x 100)" if args.workload == "c1" else "")}
        # the timed step's result against the FP64 oracle on the GPU's warps (once, outside the timed region)
        tau_g, dpart_g, _ = ctx.warp(sc.depth, sc.cams, sc.target)
        solve = pyoracle.ibr_gradient if wl["algorithm"] == 1 else pyoracle.ibr_color
        ref64, rst64 = solve(cfg, sc.views, tau_g, dpart_g, prec=0)
        vs64 = {"warps": "the GPU's (lfrv_warp_dev)", "max_rel_err": rel_err(out.cpu().numpy(), ref64),
                "iterations_gpu": stats[-1].outer_iterations, "iterations_fp64": rst64.outer_iterations}

    if rank == 0:
        line = {"metric": "views/sec to energy gap <=1e-4", "value": value, "unit": "views/s", "n_gpus": world,
                "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": sec * 1e3 / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded planes + bumps light field, no dataset)",
                "config": {"workload": wl["name"], "views": V, "input": [h, w], "target": [H, W],
                           "cg_iterations": stats[-1].outer_iterations,
                           "hole_fill_iterations": stats[-1].hole_fill_iterations, "gap": stats[-1].gap,
                           "l2": "inputs and per-step buffers exceed L2 between steps (no flush needed)",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "clocks": clocks, "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu,
                "vs_fp64": vs64,
                "e2e": {"value": e2e_value, "unit": "views/s",
                        "h2d_bytes_per_step": int(sc.views.nbytes + sc.depth.nbytes),
                        "d2h_bytes_per_step": int(3 * H * W * 4)},
                "kernels_ms_per_step": kernels_ms}
        print(json.dumps(line), flush=True)
    ctx.close()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (default per workload; c5: 5)")
    ap.add_argument("--warmup", type=int, default=None, help="untimed warm-up steps (>= 3; c5 default 3)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c5", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline and FP64 error legs")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.steps is None:
        args.steps = wl["steps"]
    args.warmup = max(3, wl["warmup"] if args.warmup is None else args.warmup)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    runner = {"c3": run_batch, "c4": run_warm, "c5": run_full, "net": run_net}.get(args.workload, run_ours)
    runner(args, rank, world)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
