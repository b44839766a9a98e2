#!/usr/bin/env python
"""Benchmark: PML slice-iterations/s on the 2048^2 x 1500-angle workload.

Workload (the reference's penalised-likelihood path, src/pml/pml_main.cc
loop): 128 slices, grid 2048 x 2048, 1500 angles uniform over [0, pi) x 2048
detector columns, 8-neighbour quadratic penalty beta = 0.05, 30 iterations
per reconstruction. Inputs are synthetic: seeded random-ellipse phantoms plus
Gaussian texture (sigma 0.02), projected by the plan's own projector, |x|
applied on upload as the PML driver does (pml_main.cc:122).

Arms
  ours (default)  the mixed-precision batched path: 16-bit lengths, 16-bit
                  gather operands (reconstruction tile, factors - 1), FP32
                  arithmetic, 8 slices per matrix pass, fused
                  backprojection+update. A "step" is one
                  iteration over all 128 slices; `value` = slice-iterations/s
                  with inputs resident on the device. Also reported: the plain
                  FP32 path (f32 lengths, one slice per pass, reference op
                  order) on a slice subset, the relative L2 error against an
                  FP64 run, the live roofline of the dominant kernel, the CPU
                  baseline (oracle port on the host cores, 1 slice-iteration),
                  and `e2e`: whole reconstructions through the C ABI with host
                  buffers (plan creation, upload, 30 iterations, download).
  --impl reference  the reference's CPU algorithm on the host cores: the
                  oracle's port of it (the reference sources cannot travel to
                  the GPU host), all host threads, one slice-iteration of the
                  same geometry per step.

Workloads (--workload): pml2048 (the default above), pml1024 (its small
case), sirt256 (SIRT 256^2 x 180 angles, 8 slices, 10 iterations, Poisson
I0=1e4), mlem1024 (MLEM 1024^2 x 720, 64 slices, 20 iterations, I0=5e3,
sinogram clipped at 1e-6), apmlr2048 (APMLR full volume: 2048 slices of
2048^2 x 1500 angles, 25 iterations, ellipsoid volume, I0=2e4) and batch64
(64 independent SIRT/MLEM problems of uneven width, angle count and slice
count, 15 iterations, advanced together one CUDA-graph launch per iteration
in waves that fit a device-memory budget).

Multi-GPU: the path is replicated, not sharded (one GPU per plan); under
torchrun every rank runs the whole workload on its GPU, value = total
slice-iterations / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("slice-iter/s at 2048²×1500 angles, mixed+batched vs plain "
          "FP32 at ≤1e-4 rel err")

WORKLOADS = {
    # the headline workload
    "pml2048": dict(alg="pml", C=2048, P=1500, S=128, iters=30, beta=0.05, texture=0.02,
                    plain_slices=8, fp64_slices=8, name=(
                        "PML 8-neighbour quadratic penalty beta=0.05, 2048x2048 grid, "
                        "128 slices, 1500 angles x 2048 columns, 30 iterations")),
    # a small case of the same kernels, for profiling captures and quick runs
    "pml1024": dict(alg="pml", C=1024, P=720, S=8, iters=30, beta=0.05, texture=0.02,
                    plain_slices=8, fp64_slices=8, name=(
                        "PML beta=0.05, 1024x1024 grid, 8 slices, 720 angles")),
    "sirt256": dict(alg="sirt", C=256, P=180, S=8, iters=10, i0=1e4,
                    plain_slices=8, fp64_slices=8, name=(
                        "SIRT, 256x256 grid, 8 slices, 180 angles x 256 columns, "
                        "10 iterations, Poisson noise I0=1e4")),
    "mlem1024": dict(alg="mlem", C=1024, P=720, S=64, iters=20, i0=5e3, clip=1e-6,
                     plain_slices=8, fp64_slices=8, name=(
                         "MLEM, 1024x1024 grid, 64 slices, 720 angles x 1024 columns, "
                         "20 iterations, Poisson noise I0=5e3, sinogram clipped at 1e-6")),
    "apmlr2048": dict(alg="apmlr", C=2048, P=1500, S=2048, iters=25, beta=0.02, i0=2e4,
                      volume=True, plain_slices=8, fp64_slices=8,
                      # the workload description asks for "acceleration on"; the
                      # reference's APMLR has no acceleration option
                      # (src/apmlr/apmlr_main.cc:20-26), so there is nothing to
                      # match and nothing is implemented under that name
                      acceleration=("not implemented: the reference's APMLR has no "
                                    "acceleration option (src/apmlr/apmlr_main.cc:20-26)"),
                      name=(
                          "APMLR 8-neighbour regulariser beta0=0.02 (beta1, delta0, "
                          "delta1, regw 1), full volume 2048 slices x 2048x2048 grid, "
                          "1500 angles x 2048 columns, 25 iterations, random-ellipsoid "
                          "volume, Poisson noise I0=2e4")),
    # uneven batch: many independent problems advanced together (tg_batch)
    "batch64": dict(
        kind="batch", alg="sirt+mlem", n=64, widths=(256, 512, 1024, 1536, 2048),
        angles=(90, 1800), slices=(1, 16), iters=15, seed=2024, name=(
            "64 independent sinograms in one CUDA-graph launch per iteration: width "
            "from {256,512,1024,1536,2048}, angles uniform in [90,1800], 1-16 slices, "
            "50/50 SIRT/MLEM, 15 iterations, grid = width")),
}


def metric_of(W):
    return METRIC if W is WORKLOADS["pml2048"] else f"slice-iter/s, {W['name']}"


def params_of(W, tg):
    return tg.default_params(W["alg"], beta=W.get("beta"))


def prep_host_sino(W, sino):
    """Host copy of the preprocessing the plan applies on upload."""
    import numpy as np
    if W["alg"] != "sirt":
        sino = np.abs(sino)
    if W.get("clip") is not None:
        sino = np.maximum(sino, np.float32(W["clip"]))
    return np.ascontiguousarray(sino, np.float32)


def host_sample_sino(W, threads):
    """One slice of the workload's data on the host (oracle projector)."""
    import numpy as np
    from oracle import oracle as O
    from trace_gb300.phantom import ellipse_phantoms, poisson_log

    C, P = W["C"], W["P"]
    theta = (np.arange(P, dtype=np.float64) * np.pi / P).astype(np.float32)
    tabs = O.angle_table(theta)
    ph = ellipse_phantoms(C, 1, seed=1234, texture_sigma=W.get("texture", 0.0))
    sino = O.forward(ph, tabs, threads=threads)
    if W.get("i0"):
        sino = poisson_log(sino, W["i0"], seed=4321, g=C)
    return tabs, prep_host_sino(W, sino)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d["hbm_gbs"], "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


class ClockSampler:
    """nvidia-smi clocks/throttle reasons while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if n_gpus > 0 else "gloo")
    return ws, rank, local


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------------------
# The reference builds MLEM and APMLR with -ffast-math (src/mlem/Makefile:11,
# src/apmlr/Makefile:11), SIRT and PML without: the CPU baseline times the
# port with the same choice.
FAST_MATH_ALGS = ("mlem", "apmlr")


def cpu_flags(alg):
    return "-O3 -ffast-math" if alg in FAST_MATH_ALGS else "-O3 (strict IEEE)"


def oracle_iteration(W, tabs, sino, threads):
    from oracle import oracle as O
    kw = {"beta": W["beta"]} if W["alg"] in ("pml", "apmlr") else {}
    fm = W["alg"] in FAST_MATH_ALGS
    O.run(W["alg"], sino, tables=tabs, n_iter=1, threads=threads, apply_abs=0,
          fast_math=fm, **kw)
    return O.port(fm).tor_last_loop_seconds()


def cpu_baseline(W, steps=1, threads=None):
    """Oracle port of the reference's threaded CPU path: 1 slice-iteration of
    the workload's geometry per step, all host threads."""
    threads = threads or os.cpu_count()
    tabs, sino = host_sample_sino(W, threads)
    secs = [oracle_iteration(W, tabs, sino, threads) for _ in range(steps)]
    C, P = W["C"], W["P"]
    return {"value": 1.0 / statistics.median(secs), "unit": "slice-iter/s",
            "cores": threads, "kind": "port",
            "sample": f"1 slice x 1 {W['alg'].upper()} iteration at {C}x{C}, {P} "
                      f"angles ({threads} threads, replicas + tree merge as the "
                      f"reference engine, {cpu_flags(W['alg'])}); median of {steps}",
            "seconds": secs}


def run_reference(args, W):
    ws, rank, _ = dist_setup(0)
    if rank != 0:
        return
    threads = os.cpu_count()
    if W.get("kind") == "batch":
        # each step: one slice-iteration of a sample of the batch's problems
        probs = batch_problems_with_theta(W)
        for _ in range(args.warmup):
            batch_cpu_baseline(W, probs)
        runs = [batch_cpu_baseline(W, probs) for _ in range(args.steps)]
        secs = [r["seconds"] / r["slice_iters"] for r in runs]
        sample = runs[0]["sample"] if runs else ""
    else:
        tabs, sino = host_sample_sino(W, threads)
        for _ in range(args.warmup):
            oracle_iteration(W, tabs, sino, threads)
        secs = [oracle_iteration(W, tabs, sino, threads) for _ in range(args.steps)]
        sample = (f"1 slice x 1 {W['alg'].upper()} iteration per step at the workload "
                  "geometry (oracle port of the reference's threaded CPU path, "
                  f"{cpu_flags(W['alg'])} as the reference builds it)")
    total = sum(secs)
    val = len(secs) / total
    line = {
        "metric": metric_of(W), "value": val, "unit": "slice-iter/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * total / len(secs), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": data_desc(W),
        "config": {"workload": W["name"], "sample": "1 slice-iteration per step"},
        "cpu_baseline": {"value": val, "unit": "slice-iter/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": "slice-iter/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def data_desc(W):
    d = ("synthetic: seeded random-ellipsoid volume" if W.get("volume")
         else "synthetic: seeded random ellipses")
    if W.get("texture"):
        d += f" + gaussian texture (sigma {W['texture']})"
    d += ", projected by the plan's projector"
    if W.get("i0"):
        d += f", Poisson counts at I0={W['i0']:g} converted with -log"
    return d


def make_data(W, device, plan):
    """Phantom -> forward projection on the device (the plan's projector) ->
    optional Poisson counting noise."""
    import torch
    from trace_gb300.phantom import (ellipse_phantoms_torch, ellipsoid_volume_torch,
                                     poisson_log_torch)

    C, S, P = W["C"], W["S"], W["P"]
    if W.get("volume"):
        ph = torch.empty((S, C, C), dtype=torch.float32, device=device)
        for z0 in range(0, S, 64):
            n = min(64, S - z0)
            ph[z0:z0 + n] = ellipsoid_volume_torch(C, S, seed=1234, device=device,
                                                   first=z0, count=n)
    else:
        ph = ellipse_phantoms_torch(C, S, seed=1234, device=device,
                                    texture_sigma=W.get("texture", 0.0))
    plan.set_recon("sirt", ph)
    del ph
    sino = torch.empty((P, S, C), dtype=torch.float32, device=device)
    plan.forward_project("sirt", out=sino)
    if W.get("i0"):
        step = max(1, (1 << 27) // (S * C))
        for a0 in range(0, P, step):
            sino[a0:a0 + step] = poisson_log_torch(sino[a0:a0 + step], W["i0"],
                                                   seed=4321 + a0, g=C)
    return sino


def upload(plan, W, sino):
    plan.set_sinogram(sino, apply_abs=W["alg"] != "sirt", clip_min=W.get("clip"))


def time_iterations(plan, alg, prm, n, stream_ptr, torch):
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(n):
        plan.iterate(alg, 1, prm)
    ev1.record()
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1)


LEN_BYTES = {"f32": 4, "bf16": 2, "f16": 2, "u16": 2}


def kernel_bytes(info, W, K, len_storage):
    """Algorithmic bytes per launch of the forward and backward kernels.

    The per-unit figure of the cached-segment-list formulation: every pass
    over one slice geometry's segments moves (4 + L) bytes per segment (int32
    pixel index + L-byte length) and serves K slices; per slice the forward
    pass adds the sinogram row read (4 P C) and one reconstruction read
    (4 g^2), the backprojection the reconstruction read and write (8 g^2)
    and, for the penalised algorithms, F and G written and read back plus
    the neighbour reads (12 g^2; APMLR's two axial neighbours 8 g^2 more).
    Summed over both kernels this is 2 Nseg (4 + L) / K + 4 P C + 12 g^2
    (+ 12 g^2 penalised) per slice-iteration.
    """
    C, P = W["C"], W["P"]
    g2 = C * C
    pen = W["alg"] in ("pml", "apmlr")
    seg = info["num_segments"] * (4 + LEN_BYTES[len_storage])
    fwd = seg + K * (4 * P * C + 4 * g2)
    back = seg + K * (8 * g2 + (12 * g2 if pen else 0)
                      + (8 * g2 if W["alg"] == "apmlr" else 0))
    return fwd, back


def format_bytes(info, W, K, tiles, half=False):
    """Bytes the kernels' own compressed matrix formats move per launch."""
    pen = W["alg"] in ("pml", "apmlr")
    fb = 2 if half and W["alg"] != "sirt" else 4  # factor bytes per ray and slice
    C, P = W["C"], W["P"]
    R, g2 = P * C, C * C
    if tiles:  # tile stream + one read of the batch + the runs' partial sums written
        fwd = info["tile_bytes"] + 4 * g2 * K + 4 * info["partial_slots"] * K
    else:      # matrix + sinogram in, factors out, batch read once
        fwd = info["forward_bytes"] + 4 * R * K * 2 + 4 * g2 * K
    back = (info["backward_bytes"] + fb * R * K + 4 * g2 * K * 2 + 4 * g2
            + (4 * g2 * K if pen else 0))
    return fwd, back


def run_ours(args, W):
    import numpy as np
    import torch

    import trace_gb300 as tg

    ws, rank, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    # every plan and every torch op of this run share one (non-default) stream
    ts = torch.cuda.Stream(device=dev)
    with torch.cuda.stream(ts):
        _run_ours(args, W, ws, rank, local, dev, ts.cuda_stream, tg, torch, np)


def _run_ours(args, W, ws, rank, local, dev, stream, tg, torch, np):
    C, P, S = W["C"], W["P"], W["S"]
    alg = W["alg"]
    theta = (np.arange(P, dtype=np.float64) * np.pi / P).astype(np.float32)
    prm = params_of(W, tg)
    K = args.slices_per_pass
    hbm_peak, peak_kind = peaks()
    t0 = time.time()
    tuned = None
    if args.autotune:
        from trace_gb300.autotune import autotune
        from trace_gb300.phantom import ellipse_phantoms_torch
        n = min(16, S)
        tp = tg.Plan(P, n, C, theta, len_storage=args.len_storage, mode="fast",
                     delta_index=True)
        tp.set_stream(stream)
        tp.set_recon("sirt", ellipse_phantoms_torch(C, n, seed=99, device=dev,
                                                    texture_sigma=W.get("texture", 0.0)))
        sample = torch.empty((P, n, C), dtype=torch.float32, device=dev)
        tp.forward_project("sirt", out=sample)
        tp.close()
        best, res = autotune(theta, sample, alg, prm, len_storage=args.len_storage,
                             stream=stream,
                             fixed={"half_gathers": True} if args.half else None)
        K, args.tiles, args.staged = (best["slices_per_pass"], best["forward_tiles"],
                                      best["backward_staged"])
        args.otf = best.get("forward_on_the_fly", False)
        args.fts = best.get("forward_tile_side", 0)
        args.btw = best.get("backward_tile_width", 0)
        args.fbw = best.get("forward_block_warps", 0)
        args.slices_per_pass = K
        tuned = {"chosen": best, "sample_slices": n,
                 "ms_per_slice_iter": [[c, round(ms, 4)] for c, ms, _, _ in res]}
        del sample

    # 16-bit gather operands need the tile-staged forward and the L1 backprojection
    args.half = args.half and args.tiles and not args.staged

    # ---- mixed-precision batched path (the measured value)
    plan = tg.Plan(P, S, C, theta, len_storage=args.len_storage, slices_per_pass=K,
                   mode="fast", delta_index=True, forward_tiles=args.tiles,
                   backward_staged=args.staged, half_gathers=args.half,
                   forward_on_the_fly=args.otf, compensated=args.compensated,
                   forward_tile_side=args.fts, backward_tile_width=args.btw,
                   batch_streams=args.batch_streams, forward_block_warps=args.fbw)
    plan.set_stream(stream)
    info = plan.info()
    sino = make_data(W, dev, plan)
    upload(plan, W, sino)
    plan.reset_recon(alg)
    # each iteration replays a captured CUDA graph (captured in the warm-up)
    plan.set_graphs(args.graphs)
    for _ in range(args.warmup):
        plan.iterate(alg, 1, prm)
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = time_iterations(plan, alg, prm, args.steps, stream, torch)
    torch.cuda.synchronize()
    barrier(ws)
    # per-kernel device times from a separate pass after the timed region
    # (the per-launch timers run eagerly, outside any graph)
    plan.set_timing(True)
    time_iterations(plan, alg, prm, max(2, min(args.steps, 3)), stream, torch)
    tim = plan.timing()
    plan.set_timing(False)
    ms_max = max_over_ranks(ms, ws)
    slice_iters = S * args.steps * ws
    value = slice_iters / (ms_max / 1000.0)
    nb = info["batches"]
    launches = args.steps * nb * (3 if args.tiles else 2)

    fwd_b, back_b = kernel_bytes(info, W, K, args.len_storage)
    fwd_f, back_f = format_bytes(info, W, K, args.tiles, args.half)
    fwd_avg = tim["forward_ms"] / max(tim["forward_launches"], 1)
    back_avg = tim["backward_ms"] / max(tim["backward_launches"], 1)
    dom = "backward" if tim["backward_ms"] >= tim["forward_ms"] else "forward"
    kname = {"forward": "k_forward_tiled" if args.tiles else "k_forward",
             "backward": "k_backward"}[dom]
    dom_bytes, dom_ms = (back_b, back_avg) if dom == "backward" else (fwd_b, fwd_avg)
    achieved = dom_bytes / (dom_ms / 1000.0) / 1e9
    traffic = ncu_traffic().get(f"{kname}:{args.workload}:{args.len_storage}:K{K}"
                                + (":half" if args.half else ""))

    def gbs(b, ms):
        return b / (ms / 1e3) / 1e9 if ms else None

    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
        "frac": achieved / hbm_peak, "peak_kind": f"{peak_kind} (burst copy)",
        "traffic": traffic, "kernel": kname,
        # the same kernel's measured DRAM bytes (ncu, one launch of this
        # configuration) over its live launch time: what HBM actually moved
        "achieved_traffic": gbs(traffic, dom_ms) if traffic else None,
        "frac_traffic": gbs(traffic, dom_ms) / hbm_peak if traffic else None,
        "algorithmic_bytes_per_launch": dom_bytes, "avg_launch_ms": dom_ms,
        "bytes_definition": "segments x (4 + L) per matrix pass + per-slice "
                            "sinogram/reconstruction/penalty bytes x K",
        "share": (tim["backward_ms"] if dom == "backward" else tim["forward_ms"]) /
                 max(tim["forward_ms"] + tim["backward_ms"], 1e-9),
        "kernels": {
            ("k_forward_tiled" if args.tiles else "k_forward"): {
                "avg_ms": fwd_avg, "bytes": fwd_b, "gbs": gbs(fwd_b, fwd_avg),
                "format_bytes": fwd_f, "format_gbs": gbs(fwd_f, fwd_avg)},
            "k_fwd_finish": {"avg_ms": tim["other_ms"] / max(tim["other_launches"], 1),
                             "format_bytes": 4 * info["partial_slots"] * K
                                             + 4 * W["P"] * W["C"] * K * 2},
            "k_backward": {"avg_ms": back_avg, "bytes": back_b, "gbs": gbs(back_b, back_avg),
                           "format_bytes": back_f, "format_gbs": gbs(back_f, back_avg)},
        },
    }

    recon_bytes = 4 * S * C * C
    sino_bytes = 4 * P * S * C
    plan.close()  # before the comparison plans (a full volume holds ~200 GB)
    del plan
    torch.cuda.empty_cache()

    # relative L2 against an FP64 run on a slice subset
    rel = None
    if args.fp64_check and rank == 0:
        rel = fp64_check(args, W, theta, sino, prm, tg, torch, dev)

    # ---- FP32 on the measured schedule, and the plain FP32 path (f32
    # lengths, 1 slice per pass, reference operation order)
    plain = same = None
    if args.plain and rank == 0:
        same = fp32_same_schedule(args, W, theta, sino, prm, tg, torch, stream)
        torch.cuda.empty_cache()
        plain = plain_path(args, W, theta, sino, prm, tg, torch, stream)

    # ---- end to end through the C ABI with host buffers
    e2e = None
    if args.e2e and rank == 0:
        e2e = end_to_end(args, W, theta, sino, prm, tg, torch, stream)
    del sino
    torch.cuda.empty_cache()

    cpu = None
    if args.cpu_baseline and rank == 0 and ws == 1:
        cpu = cpu_baseline(W)

    if rank != 0:
        return
    line = {
        "metric": metric_of(W), "value": value, "unit": "slice-iter/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": f"f32 arithmetic, {args.len_storage} segment lengths",
        "data": data_desc(W),
        "config": {"workload": W["name"], "slices_per_pass": K,
                   "len_storage": args.len_storage, "index": "4-bit delta",
                   "gather_operands": "f16 (tile, factor-1)" if args.half else "f32",
                   "intersections": "traced on the fly" if args.otf else "cached",
                   "forward": (f"tile-staged ({args.fts or 64}x{args.fts or 64} "
                               "shared-memory tiles)") if args.tiles else "ray-ordered",
                   "backward_tile": {4: "4x8", 16: "16x2"}.get(args.btw, "8x4") + " pixels",
                   "forward_block_warps": args.fbw or 32,
                   "step": f"one {alg.upper()} iteration over all {S} slices",
                   "graphs": bool(args.graphs),
                   "batch_streams": args.batch_streams,
                   **({"acceleration": W["acceleration"]} if W.get("acceleration") else {}),
                   "summation": "compensated (Kahan over 8-segment / 4-angle blocks)"
                                if args.compensated else "FMA chains",
                   "l2": "inputs larger than L2 (system matrix "
                         f"{(info['forward_bytes'] + info['backward_bytes']) / 1e9:.1f} GB "
                         "streamed per step)",
                   "parallelism": f"replicas x{ws}"},
        "roofline": roofline, "clocks": clk.summary(), "gpu_launches": launches,
        "setup_ms": info["setup_ms"], "num_segments_per_slice": info["num_segments"],
        "device_bytes": info["device_bytes"],
        "rel_l2_vs_fp64": rel, "plain_fp32": plain, "fp32_same_schedule": same,
        "mixed_vs_fp32_same_schedule": value / same["value"] if same else None,
        "mixed_vs_plain_fp32": value / plain["value"] if plain else None,
        "e2e": e2e, "autotune": tuned,
        "cpu_baseline": cpu,
        "wall_s": time.time() - t0,
    }
    print(json.dumps(line), flush=True)


def fp64_slice_subset(W):
    """Indices of the slices the FP64 comparison runs: spread evenly over the
    volume for the slice-independent algorithms; for APMLR, whose slices are
    coupled by the axial penalty, one contiguous block from the middle (run
    as its own sub-volume by every configuration compared)."""
    import numpy as np
    n, S = W["fp64_slices"], W["S"]
    if n >= S:
        return list(range(S))
    if W["alg"] == "apmlr":
        s0 = (S - n) // 2
        return list(range(s0, s0 + n))
    return sorted(set(int(round(x)) for x in np.linspace(0, S - 1, n)))


def fp64_check(args, W, theta, sino, prm, tg, torch, dev):
    """Per-iteration relative L2 against the GPU FP64 mode on a slice subset
    (fp64_slice_subset), over the workload's full iteration count, for the
    mixed path as measured (its arithmetic per slice does not depend on the
    slices per pass), the FP32 path on the same schedule (f32 lengths and
    gather operands, same slices per pass and forward) and the plain FP32
    path (the reference's operation order)."""
    import numpy as np
    idx = fp64_slice_subset(W)
    n = len(idx)
    sub = sino[:, idx, :].contiguous()
    configs = {
        "fp64": dict(len_storage="f32", mode="fp64"),
        # the measured configuration, same kernels (same slices per pass: the
        # subset fills one batch)
        "mixed": dict(len_storage=args.len_storage, mode="fast", delta_index=True,
                      forward_tiles=args.tiles, backward_staged=args.staged,
                      half_gathers=args.half, slices_per_pass=args.slices_per_pass,
                      compensated=args.compensated, forward_tile_side=args.fts,
                      backward_tile_width=args.btw, forward_block_warps=args.fbw),
        "fp32_same_schedule": dict(len_storage="f32", mode="fast", delta_index=True,
                                   forward_tiles=args.tiles, backward_staged=args.staged,
                                   slices_per_pass=args.slices_per_pass,
                                   backward_tile_width=args.btw,
                                   compensated=args.compensated),
        "plain_fp32": dict(len_storage="f32", mode="exact"),
    }
    runs = {}
    alg = W["alg"]
    for key, kw in configs.items():
        p = tg.Plan(W["P"], n, W["C"], theta, **kw)
        p.set_stream(torch.cuda.current_stream().cuda_stream)
        upload(p, W, sub)
        p.reset_recon(alg)
        snaps = []
        for _ in range(W["iters"]):
            p.iterate(alg, 1, prm)
            snaps.append(p.get_recon(alg))
        runs[key] = snaps
        p.close()
        torch.cuda.empty_cache()
    out = {"slices": n, "slice_indices": idx, "iterations": W["iters"],
           "reference": "GPU FP64 mode (pinned to the CPU FP64 oracle by the -m gpu tests)"}
    for key in ("mixed", "fp32_same_schedule", "plain_fp32"):
        errs = [float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b))
                for a, b in zip(runs[key], runs["fp64"])]
        out[key] = {"max": max(errs), "final": errs[-1], "per_iteration": errs}
    return out


def fp32_same_schedule(args, W, theta, sino, prm, tg, torch, stream):
    """The FP32 GPU path on the measured schedule: f32 lengths and FP32
    gather operands, with the same slices per pass, forward projection,
    backprojection and CUDA graphs as the mixed path, over the workload's
    slices (at most 256 of a full volume)."""
    n = min(W["S"], 256)
    sub = sino[:, :n, :].contiguous() if n < W["S"] else sino
    p = tg.Plan(W["P"], n, W["C"], theta, len_storage="f32",
                slices_per_pass=args.slices_per_pass, mode="fast", delta_index=True,
                forward_tiles=args.tiles, backward_staged=args.staged,
                forward_on_the_fly=args.otf, backward_tile_width=args.btw)
    p.set_stream(stream)
    p.set_graphs(True)
    info = p.info()
    alg = W["alg"]
    upload(p, W, sub)
    p.reset_recon(alg)
    for _ in range(args.warmup):
        p.iterate(alg, 1, prm)
    torch.cuda.synchronize()
    ms = time_iterations(p, alg, prm, args.steps, stream, torch)
    p.close()
    return {"value": n * args.steps / (ms / 1000.0), "unit": "slice-iter/s",
            "slices": n, "steps": args.steps, "setup_ms": info["setup_ms"],
            "matrix_bytes": info["forward_bytes"] + info["backward_bytes"] + info["tile_bytes"],
            "config": f"f32 lengths, FP32 gather operands, {args.slices_per_pass} slices "
                      "per pass, " + ("tile-staged forward" if args.tiles else
                                      "ray-ordered forward") + ", CUDA graphs"}


def plain_path(args, W, theta, sino, prm, tg, torch, stream):
    """The plain FP32 path in the reference's operation order: f32 lengths,
    int32 indices, one slice per matrix pass, exact arithmetic."""
    n = W["plain_slices"]
    sub = sino[:, :n, :].contiguous()
    p = tg.Plan(W["P"], n, W["C"], theta, len_storage="f32", slices_per_pass=1,
                mode="exact")
    p.set_stream(stream)
    info = p.info()
    alg = W["alg"]
    upload(p, W, sub)
    p.reset_recon(alg)
    for _ in range(max(1, args.warmup // 2)):
        p.iterate(alg, 1, prm)
    torch.cuda.synchronize()
    steps = max(2, args.steps // 2)
    ms = time_iterations(p, alg, prm, steps, stream, torch)
    p.close()
    return {"value": n * steps / (ms / 1000.0), "unit": "slice-iter/s",
            "slices": n, "steps": steps, "setup_ms": info["setup_ms"],
            "matrix_bytes": info["forward_bytes"] + info["backward_bytes"],
            "config": "reference operation order: f32 lengths, explicit int32 indices, "
                      "1 slice per pass, IEEE-rounded mul/add/div"}


def end_to_end(args, W, theta, sino, prm, tg, torch, stream):
    """Whole reconstructions through the C ABI: plan creation (tracing),
    sinogram upload from pinned host memory, iterations, download."""
    import numpy as np
    host_sino = sino.cpu().pin_memory()
    host = host_sino.numpy()
    halo = 1 if W["alg"] == "apmlr" else 0
    # the reconstruction lands in pinned host memory, as the sinogram leaves it
    out = torch.empty((W["S"] + 2 * halo, W["C"], W["C"]), dtype=torch.float32).pin_memory()
    times = []
    for i in range(args.e2e_warmup + args.e2e_steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        p = tg.Plan(W["P"], W["S"], W["C"], theta, len_storage=args.len_storage,
                    slices_per_pass=args.slices_per_pass, mode="fast",
                    delta_index=True, forward_tiles=args.tiles,
                    backward_staged=args.staged, half_gathers=args.half,
                    forward_on_the_fly=args.otf, compensated=args.compensated,
                    forward_tile_side=args.fts, backward_tile_width=args.btw,
                    batch_streams=args.batch_streams, forward_block_warps=args.fbw)
        p.set_stream(stream)
        p.set_graphs(args.graphs)
        upload(p, W, host)
        p.reset_recon(W["alg"])
        # the iterations, then the reconstruction into the pinned buffer (the
        # last iteration's slice batches leave as each one finishes)
        p.iterate(W["alg"], W["iters"], prm, out=out)
        p.synchronize()
        dt = time.perf_counter() - t
        p.close()
        if i >= args.e2e_warmup:
            times.append(dt)
    per = statistics.median(times)
    return {"value": W["S"] * W["iters"] / per, "unit": "slice-iter/s",
            "h2d_bytes_per_step": int(host.nbytes),
            "d2h_bytes_per_step": int(out.numel() * 4),
            "step": f"plan creation + upload + {W['iters']} iterations + download "
                    "(tg_iterate_get_recon)",
            "seconds_per_step": per, "steps": len(times)}


def batch_problems(W):
    import numpy as np
    rng = np.random.default_rng(W["seed"])
    n = W["n"]
    C = rng.choice(W["widths"], n)
    P = rng.integers(W["angles"][0], W["angles"][1] + 1, n)
    S = rng.integers(W["slices"][0], W["slices"][1] + 1, n)
    algs = rng.permutation(["sirt"] * (n // 2) + ["mlem"] * (n - n // 2))
    return [dict(C=int(c), P=int(p), S=int(s), alg=str(a))
            for c, p, s, a in zip(C, P, S, algs)]


def batch_problems_with_theta(W):
    import numpy as np
    probs = batch_problems(W)
    for pr in probs:
        pr["theta"] = (np.arange(pr["P"], dtype=np.float64) * np.pi / pr["P"]).astype(np.float32)
    return probs


def batch_plan_kw(pr, args, tuned=None):
    """Plan options of one batch problem: 16-bit lengths, tile-staged forward,
    slices per pass the largest power of two <= min(8, slices), and the tile
    side and backprojection tile shape autotuned for its detector width."""
    K = 1
    while K * 2 <= min(8, pr["S"]):
        K *= 2
    kw = dict(len_storage="u16", slices_per_pass=K, mode="fast", delta_index=True,
              forward_tiles=True, half_gathers=args.half)
    if tuned and pr["C"] in tuned:
        kw.update(tuned[pr["C"]])
    return kw


def batch_autotune(args, probs, hosts, stream):
    """Per detector width: the forward tile side and backprojection tile shape
    that the autotuner measures fastest on that width's problem with the most
    angles (its slices, its algorithm)."""
    from trace_gb300.autotune import autotune
    tuned, log = {}, {}
    for C in sorted(set(pr["C"] for pr in probs)):
        i = max((j for j, pr in enumerate(probs) if pr["C"] == C),
                key=lambda j: probs[j]["P"])
        pr = probs[i]
        kw = batch_plan_kw(pr, args)
        best, res = autotune(pr["theta"], hosts[i], pr["alg"], len_storage="u16",
                             space={"slices_per_pass": (kw["slices_per_pass"],),
                                    "forward_tiles": (True,)},
                             fixed={"half_gathers": args.half}, stream=stream)
        tuned[C] = {k: best[k] for k in ("forward_tile_side", "backward_tile_width")
                    if k in best}
        log[str(C)] = {"problem": i, "chosen": tuned[C],
                       "ms_per_slice_iter": [[c, round(ms, 4)] for c, ms, _, _ in res]}
    return tuned, log


def batch_estimate_bytes(pr):
    """Device bytes of one problem's plan (matrices, tile stream, buffers)."""
    C, P, S = pr["C"], pr["P"], pr["S"]
    seg = 1.2 * C * C * P
    return seg * 5.5 + ((P + 3) // 4 * 4) * C * C * 4 + 16 * C * C * (S + 8) + 12 * P * C * (S + 8)


def run_batch(args, W):
    import numpy as np
    import torch

    import trace_gb300 as tg
    from trace_gb300.phantom import ellipse_phantoms_torch

    ws, rank, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ts = torch.cuda.Stream(device=dev)
    hbm_peak, peak_kind = peaks()
    t_start = time.time()
    probs = batch_problems_with_theta(W)
    with torch.cuda.stream(ts):
        stream = ts.cuda_stream
        # inputs: phantom -> projection on the device, kept in pinned host memory
        hosts = []
        for i, pr in enumerate(probs):
            gp = tg.Plan(pr["P"], pr["S"], pr["C"], pr["theta"], mode="fast")
            gp.set_stream(stream)
            gp.set_recon("sirt", ellipse_phantoms_torch(pr["C"], pr["S"], seed=1000 + i,
                                                        device=dev))
            sino = torch.empty((pr["P"], pr["S"], pr["C"]), dtype=torch.float32, device=dev)
            gp.forward_project("sirt", out=sino)
            gp.close()
            hosts.append(sino.cpu().pin_memory())
            del sino
        # reconstructions land in pinned host memory, as the sinograms leave it
        outs_host = [torch.empty((pr["S"], pr["C"], pr["C"]), dtype=torch.float32).pin_memory()
                     for pr in probs]
        torch.cuda.synchronize()
        tuned, tune_log = (batch_autotune(args, probs, hosts, stream) if args.autotune
                           else (None, None))
        args.batch_tuned = tuned
        budget = args.batch_budget_gb * 1e9
        waves, cur, used = [], [], 0.0
        for i, pr in enumerate(probs):
            b = batch_estimate_bytes(pr)
            if cur and used + b > budget:
                waves.append(cur)
                cur, used = [], 0.0
            cur.append(i)
            used += b
        waves.append(cur)
        iters = W["iters"]
        e2e_s = iter_ms = setup_ms = alg_bytes = fmt_traffic = 0.0
        ratios = ncu_traffic()
        timed_slice_iters = launches = h2d = d2h = 0
        multi = True
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            for wave in waves:
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                plans = []
                for i in wave:
                    pr = probs[i]
                    p = tg.Plan(pr["P"], pr["S"], pr["C"], pr["theta"],
                                **batch_plan_kw(pr, args, tuned))
                    p.set_stream(stream)
                    p.set_sinogram(hosts[i], apply_abs=pr["alg"] != "sirt")
                    p.reset_recon(pr["alg"])
                    plans.append(p)
                    setup_ms += p.info()["setup_ms"]
                    h2d += hosts[i].numel() * 4
                algs = [probs[i]["alg"] for i in wave]
                batch = tg.Batch(plans)
                batch.iterate(algs, 1)  # first iteration: captures its graph
                ev0.record()
                batch.iterate(algs, iters - 1)
                ev1.record()
                binfo = batch.info()
                multi = multi and binfo["multi"]
                outs = [p.get_recon(probs[i]["alg"], out=outs_host[i])
                        for p, i in zip(plans, wave)]
                torch.cuda.synchronize()
                e2e_s += time.perf_counter() - t0
                iter_ms += ev0.elapsed_time(ev1)
                for p, i in zip(plans, wave):
                    pr = probs[i]
                    info = p.info()
                    timed_slice_iters += pr["S"] * (iters - 1)
                    K = batch_plan_kw(pr, args, tuned)["slices_per_pass"]
                    Wp = dict(C=pr["C"], P=pr["P"], alg=pr["alg"])
                    fb, bb = kernel_bytes(info, Wp, K, "u16")
                    alg_bytes += (iters - 1) * info["batches"] * (fb + bb)
                    ff, bf = format_bytes(info, Wp, K, True, args.half)
                    fin = 4 * info["partial_slots"] * K + 4 * pr["P"] * pr["C"] * K * 2
                    fmt_traffic += (iters - 1) * info["batches"] * (
                        ff * ratios.get("ratio:k_forward_tiled", 1.0)
                        + fin * ratios.get("ratio:k_fwd_finish", 1.0)
                        + bf * ratios.get("ratio:k_backward", 1.0))
                d2h += sum(o.numel() * 4 for o in outs)
                launches += (iters - 1) * binfo["launches"]
                batch.close()
                for p in plans:
                    p.close()
                del plans, outs
    ms_max = max_over_ranks(iter_ms, ws)
    value = timed_slice_iters * ws / (ms_max / 1e3)
    total_slice_iters = sum(pr["S"] for pr in probs) * W["iters"]
    achieved = alg_bytes / (iter_ms / 1e3) / 1e9
    rel = None
    if args.fp64_check and rank == 0:
        with torch.cuda.stream(ts):
            rel = batch_fp64_check(args, W, probs, hosts, outs_host, tg, torch, ts.cuda_stream)
    cpu = None
    if args.cpu_baseline and rank == 0 and ws == 1:
        cpu = batch_cpu_baseline(W, probs)
    if rank != 0:
        return
    line = {
        "metric": metric_of(W), "value": value, "unit": "slice-iter/s",
        "n_gpus": args.gpus, "steps": iters - 1, "warmup": 1,
        "ms_per_step": iter_ms / (iters - 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 arithmetic, u16 segment lengths"
                 + (", f16 gather operands" if args.half else ""),
        "data": "synthetic: seeded random ellipses projected by the plan's projector",
        "config": {"workload": W["name"], "problems": len(probs),
                   "waves": len(waves), "wave_budget_gb": args.batch_budget_gb,
                   "step": ("one iteration of every problem of a wave: one CUDA graph of "
                            "multi-plan launches (per slice-batch round, one launch per "
                            "kernel variant whose blocks walk all problems' tiles and rays)")
                           if multi else
                           ("one iteration of every problem of a wave, one CUDA-graph launch "
                            "(plans forked over up to 16 streams inside the graph)"),
                   "multi_plan_launches": multi,
                   "slices_per_pass": "largest power of two <= min(8, slices)",
                   "l2": "inputs larger than L2 (system matrices streamed per step)",
                   "parallelism": f"replicas x{ws}"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                     "unit": "GB/s", "frac": achieved / hbm_peak,
                     "peak_kind": f"{peak_kind} (burst copy)",
                     "traffic": fmt_traffic / (iters - 1),
                     "traffic_basis": "DRAM bytes per step (one iteration of every wave): "
                                      "each kernel's format bytes times its measured "
                                      "DRAM/format ratio (profiles/ncu_traffic.json)",
                     "frac_traffic": fmt_traffic / (iter_ms / 1e3) / 1e9 / hbm_peak,
                     "kernel": "all kernels of the batch (whole-step effective bandwidth)"},
        "clocks": clk.summary(), "gpu_launches": launches,
        "setup_ms": setup_ms, "rel_l2_vs_fp64": rel, "autotune": tune_log,
        "e2e": {"value": total_slice_iters / e2e_s, "unit": "slice-iter/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "step": "every wave: plan creation (tracing), upload from pinned host, "
                        f"{iters} iterations, download", "seconds": e2e_s},
        "cpu_baseline": cpu, "wall_s": time.time() - t_start,
    }
    print(json.dumps(line), flush=True)


def batch_fp64_check(args, W, probs, hosts, outs_host, tg, torch, stream, sample=8):
    """Relative L2 against the GPU FP64 mode for a seeded sample of the
    batch's problems: per iteration, from a plan with the batch's
    configuration iterated alone (the multi-plan launches give its results
    bit for bit), and for the final reconstruction the batch delivered."""
    import numpy as np
    rng = np.random.default_rng(W["seed"] + 2)
    idx = sorted(rng.choice(len(probs), sample, replace=False).tolist())
    out = {"problems": [], "reference": "GPU FP64 mode", "iterations": W["iters"]}
    worst = 0.0
    for i in idx:
        pr = probs[i]
        runs = {}
        for key, kw in (("fp64", dict(len_storage="f32", mode="fp64")),
                        ("mixed", batch_plan_kw(pr, args, getattr(args, "batch_tuned", None)))):
            p = tg.Plan(pr["P"], pr["S"], pr["C"], pr["theta"], **kw)
            p.set_stream(stream)
            p.set_sinogram(hosts[i], apply_abs=pr["alg"] != "sirt")
            p.reset_recon(pr["alg"])
            snaps = []
            for _ in range(W["iters"]):
                p.iterate(pr["alg"], 1)
                snaps.append(p.get_recon(pr["alg"]))
            runs[key] = snaps
            p.close()
        errs = [float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b))
                for a, b in zip(runs["mixed"], runs["fp64"])]
        final_batch = outs_host[i].numpy()
        eb = float(np.linalg.norm(final_batch.astype(np.float64) - runs["fp64"][-1])
                   / np.linalg.norm(runs["fp64"][-1]))
        worst = max(worst, max(errs), eb)
        out["problems"].append({"index": i, "alg": pr["alg"], "C": pr["C"], "P": pr["P"],
                                "S": pr["S"], "max": max(errs), "final": errs[-1],
                                "batch_final": eb})
        torch.cuda.empty_cache()
    out["max"] = worst
    return out


def batch_cpu_baseline(W, probs, sample=4):
    """The oracle port on a sample of the batch's problems: one slice-iteration
    of each sampled geometry, all host threads."""
    import numpy as np
    from oracle import oracle as O
    from trace_gb300.phantom import ellipse_phantoms
    threads = os.cpu_count()
    rng = np.random.default_rng(W["seed"] + 1)
    idx = sorted(rng.choice(len(probs), sample, replace=False).tolist())
    secs = 0.0
    for i in idx:
        pr = probs[i]
        tabs = O.angle_table(pr["theta"])
        sino = O.forward(ellipse_phantoms(pr["C"], 1, seed=1000 + i), tabs, threads=threads)
        if pr["alg"] != "sirt":
            sino = np.abs(sino)
        fm = pr["alg"] in FAST_MATH_ALGS
        O.run(pr["alg"], sino, tables=tabs, n_iter=1, threads=threads, fast_math=fm)
        secs += O.port(fm).tor_last_loop_seconds()
    return {"value": sample / secs, "unit": "slice-iter/s", "cores": threads,
            "kind": "port", "seconds": secs, "slice_iters": sample,
            "sample": "1 slice-iteration of each of the problems " + ", ".join(
                f"{probs[i]['alg']} {probs[i]['C']} columns x {probs[i]['P']} angles"
                for i in idx)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="pml2048", choices=sorted(WORKLOADS))
    ap.add_argument("--len-storage", default="u16", choices=["u16", "f16", "bf16", "f32"])
    ap.add_argument("--slices-per-pass", type=int, default=8)
    ap.add_argument("--no-tiles", dest="tiles", action="store_false",
                    help="ray-ordered forward projection instead of the tile-staged one")
    ap.add_argument("--staged", action="store_true",
                    help="shared-memory-staged backprojection")
    ap.add_argument("--no-half-gathers", dest="half", action="store_false",
                    help="FP32 gather operands instead of halves (shared-memory "
                         "tile, ratio factors)")
    ap.add_argument("--on-the-fly", dest="otf", action="store_true",
                    help="no stored ray-ordered forward matrix: rays traced during "
                         "forward projections")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="skip timing the plan configurations on a 16-slice sample "
                         "(run the defaults or the flags given)")
    ap.add_argument("--forward-tile-side", dest="fts", type=int, default=0,
                    help="forward tile side (32, 64, 96; 0 = the plan default)")
    ap.add_argument("--forward-block-warps", dest="fbw", type=int, default=0,
                    help="warps per forward tile block (8, 16, 32; 0 = the plan default)")
    ap.add_argument("--backward-tile-width", dest="btw", type=int, default=0,
                    help="backprojection tile width (4, 8, 16; 0 = the plan default)")
    ap.add_argument("--compensated", action="store_true",
                    help="compensated (Kahan) ray and pixel sums in the measured path")
    ap.add_argument("--batch-streams", type=int, default=0,
                    help="1: every slice batch on one stream; 2 (0 = default): odd "
                         "batches on a second stream")
    ap.add_argument("--no-graphs", dest="graphs", action="store_false",
                    help="eager launches instead of one CUDA graph per iteration")
    ap.add_argument("--no-plain", dest="plain", action="store_false")
    ap.add_argument("--no-e2e", dest="e2e", action="store_false")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-fp64-check", dest="fp64_check", action="store_false")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--e2e-warmup", type=int, default=1)
    ap.add_argument("--batch-budget-gb", type=float, default=200.0,
                    help="batch64: device memory of the plans advanced together")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("note: fewer than 3 warm-up steps", file=sys.stderr)
    W = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, W)
    elif W.get("kind") == "batch":
        run_batch(args, W)
    else:
        run_ours(args, W)


if __name__ == "__main__":
    main()
