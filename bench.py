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
    "pml2048": dict(C=2048, P=1500, S=128, iters=30, beta=0.05, texture=0.02,
                    plain_slices=8, fp64_slices=1, name=(
                        "PML 8-neighbour quadratic penalty beta=0.05, 2048x2048 grid, "
                        "128 slices, 1500 angles x 2048 columns, 30 iterations")),
    # a small case of the same kernels, for profiling captures and quick runs
    "pml1024": dict(C=1024, P=720, S=8, iters=30, beta=0.05, texture=0.02,
                    plain_slices=8, fp64_slices=1, name=(
                        "PML beta=0.05, 1024x1024 grid, 8 slices, 720 angles")),
}


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
def cpu_baseline(W, steps=1, threads=None):
    """Oracle port of the reference's threaded CPU path: 1 slice-iteration of
    the workload's geometry per step, all host threads."""
    import numpy as np
    from oracle import oracle as O
    from trace_gb300.phantom import ellipse_phantoms

    C, P = W["C"], W["P"]
    threads = threads or os.cpu_count()
    theta = (np.arange(P, dtype=np.float64) * np.pi / P).astype(np.float32)
    tabs = O.angle_table(theta)
    ph = ellipse_phantoms(C, 1, seed=1234, texture_sigma=W["texture"])
    sino = O.forward(ph, tabs, threads=threads)
    secs = []
    for _ in range(steps):
        O.run("pml", sino, tables=tabs, n_iter=1, beta=W["beta"], threads=threads)
        secs.append(O.port().tor_last_loop_seconds())
    return {"value": 1.0 / statistics.median(secs), "unit": "slice-iter/s",
            "cores": threads, "kind": "port",
            "sample": f"1 slice x 1 PML iteration at {C}x{C}, {P} angles "
                      f"({threads} threads, replicas + tree merge as the "
                      f"reference engine); median of {steps}",
            "seconds": secs}


def run_reference(args, W):
    ws, rank, _ = dist_setup(0)
    if rank != 0:
        return
    import numpy as np
    from oracle import oracle as O
    from trace_gb300.phantom import ellipse_phantoms

    C, P = W["C"], W["P"]
    threads = os.cpu_count()
    theta = (np.arange(P, dtype=np.float64) * np.pi / P).astype(np.float32)
    tabs = O.angle_table(theta)
    ph = ellipse_phantoms(C, 1, seed=1234, texture_sigma=W["texture"])
    sino = O.forward(ph, tabs, threads=threads)
    for _ in range(args.warmup):
        O.run("pml", sino, tables=tabs, n_iter=1, beta=W["beta"], threads=threads)
    secs = []
    for _ in range(args.steps):
        O.run("pml", sino, tables=tabs, n_iter=1, beta=W["beta"], threads=threads)
        secs.append(O.port().tor_last_loop_seconds())
    total = sum(secs)
    val = len(secs) / total
    line = {
        "metric": METRIC, "value": val, "unit": "slice-iter/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * total / len(secs), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded random ellipses + gaussian texture",
        "config": {"workload": W["name"], "sample": "1 slice-iteration per step"},
        "cpu_baseline": {"value": val, "unit": "slice-iter/s", "cores": threads,
                         "kind": "port",
                         "sample": "1 slice x 1 PML iteration per step at the "
                                   "workload geometry (oracle port of the "
                                   "reference's threaded CPU path)"},
        "e2e": {"value": val, "unit": "slice-iter/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def make_data(W, device, plan):
    """Phantom -> forward projection on the device (the plan's projector)."""
    import torch
    from trace_gb300.phantom import ellipse_phantoms_torch

    C, S = W["C"], W["S"]
    ph = ellipse_phantoms_torch(C, S, seed=1234, device=device,
                                texture_sigma=W["texture"])
    plan.set_recon("sirt", ph)
    sino = torch.empty((W["P"], S, C), dtype=torch.float32, device=device)
    plan.forward_project("sirt", out=sino)
    del ph
    return sino


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


def kernel_bytes(info, W, K, len_storage, pen=True):
    """Algorithmic bytes per launch of the forward and backward kernels.

    The per-unit figure of the cached-segment-list formulation: every pass
    over one slice geometry's segments moves (4 + L) bytes per segment (int32
    pixel index + L-byte length) and serves K slices; per slice the forward
    pass adds the sinogram row read (4 P C) and one reconstruction read
    (4 g^2), the backprojection the reconstruction read and write (8 g^2)
    and, for the penalised algorithms, F and G written and read back plus
    the neighbour reads (12 g^2). Summed over both kernels this is
    2 Nseg (4 + L) / K + 4 P C + 12 g^2 + 12 g^2 per slice-iteration.
    """
    C, P = W["C"], W["P"]
    g2 = C * C
    seg = info["num_segments"] * (4 + LEN_BYTES[len_storage])
    fwd = seg + K * (4 * P * C + 4 * g2)
    back = seg + K * (8 * g2 + (12 * g2 if pen else 0))
    return fwd, back


def format_bytes(info, W, K, tiles, pen=True):
    """Bytes the kernels' own compressed matrix formats move per launch."""
    C, P = W["C"], W["P"]
    R, g2 = P * C, C * C
    if tiles:  # tile stream + one read of the batch + the ray sums written
        fwd = info["tile_bytes"] + 4 * g2 * K + 4 * R * K
    else:      # matrix + sinogram in, factors out, batch read once
        fwd = info["forward_bytes"] + 4 * R * K * 2 + 4 * g2 * K
    back = (info["backward_bytes"] + 4 * R * K + 4 * g2 * K * 2 + 4 * g2
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
    theta = (np.arange(P, dtype=np.float64) * np.pi / P).astype(np.float32)
    prm = tg.default_params("pml", beta=W["beta"])
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
                                                    texture_sigma=W["texture"]))
        sample = torch.empty((P, n, C), dtype=torch.float32, device=dev)
        tp.forward_project("sirt", out=sample)
        tp.close()
        best, res = autotune(theta, sample, "pml", prm, len_storage=args.len_storage,
                             stream=stream)
        K, args.tiles, args.staged = (best["slices_per_pass"], best["forward_tiles"],
                                      best["backward_staged"])
        args.slices_per_pass = K
        tuned = {"chosen": best, "sample_slices": n,
                 "ms_per_slice_iter": [[c, round(ms, 4)] for c, ms, _ in res]}
        del sample

    # 16-bit gather operands need the tile-staged forward and the L1 backprojection
    args.half = args.half and args.tiles and not args.staged

    # ---- mixed-precision batched path (the measured value)
    plan = tg.Plan(P, S, C, theta, len_storage=args.len_storage, slices_per_pass=K,
                   mode="fast", delta_index=True, forward_tiles=args.tiles,
                   backward_staged=args.staged, half_gathers=args.half)
    plan.set_stream(stream)
    info = plan.info()
    sino = make_data(W, dev, plan)
    plan.set_sinogram(sino, apply_abs=True)
    plan.reset_recon("pml")
    for _ in range(args.warmup):
        plan.iterate("pml", 1, prm)
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    plan.set_timing(True)
    with ClockSampler(local) as clk:
        ms = time_iterations(plan, "pml", prm, args.steps, stream, torch)
    torch.cuda.synchronize()
    barrier(ws)
    tim = plan.timing()
    plan.set_timing(False)
    ms_max = max_over_ranks(ms, ws)
    slice_iters = S * args.steps * ws
    value = slice_iters / (ms_max / 1000.0)
    nb = info["batches"]
    launches = args.steps * nb * (3 if args.tiles else 2)

    fwd_b, back_b = kernel_bytes(info, W, K, args.len_storage)
    fwd_f, back_f = format_bytes(info, W, K, args.tiles)
    fwd_avg = tim["forward_ms"] / max(tim["forward_launches"], 1)
    back_avg = tim["backward_ms"] / max(tim["backward_launches"], 1)
    dom = "backward" if tim["backward_ms"] >= tim["forward_ms"] else "forward"
    kname = {"forward": "k_forward_tiled" if args.tiles else "k_forward",
             "backward": "k_backward"}[dom]
    dom_bytes, dom_ms = (back_b, back_avg) if dom == "backward" else (fwd_b, fwd_avg)
    achieved = dom_bytes / (dom_ms / 1000.0) / 1e9
    traffic = ncu_traffic().get(f"{kname}:{args.workload}:{args.len_storage}:K{K}")

    def gbs(b, ms):
        return b / (ms / 1e3) / 1e9 if ms else None

    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
        "frac": achieved / hbm_peak, "peak_kind": f"{peak_kind} (burst copy)",
        "traffic": traffic, "kernel": kname,
        "algorithmic_bytes_per_launch": dom_bytes, "avg_launch_ms": dom_ms,
        "bytes_definition": "segments x (4 + L) per matrix pass + per-slice "
                            "sinogram/reconstruction/penalty bytes x K",
        "share": (tim["backward_ms"] if dom == "backward" else tim["forward_ms"]) /
                 max(tim["forward_ms"] + tim["backward_ms"], 1e-9),
        "kernels": {
            ("k_forward_tiled" if args.tiles else "k_forward"): {
                "avg_ms": fwd_avg, "bytes": fwd_b, "gbs": gbs(fwd_b, fwd_avg),
                "format_bytes": fwd_f, "format_gbs": gbs(fwd_f, fwd_avg)},
            "k_fwd_finish": {"avg_ms": tim["other_ms"] / max(tim["other_launches"], 1)},
            "k_backward": {"avg_ms": back_avg, "bytes": back_b, "gbs": gbs(back_b, back_avg),
                           "format_bytes": back_f, "format_gbs": gbs(back_f, back_avg)},
        },
    }

    # relative L2 against an FP64 run on a slice subset
    rel = None
    if args.fp64_check and rank == 0:
        rel = fp64_check(args, W, theta, sino, prm, tg, torch, dev)

    recon_bytes = 4 * S * C * C
    sino_bytes = 4 * P * S * C
    plan.close()
    del plan

    # ---- plain FP32 path (f32 lengths, 1 slice per pass, reference op order)
    plain = None
    if args.plain and rank == 0:
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
        "metric": METRIC, "value": value, "unit": "slice-iter/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": f"f32 arithmetic, {args.len_storage} segment lengths",
        "data": "synthetic: seeded random ellipses + gaussian texture (sigma 0.02), "
                "projected by the plan's projector",
        "config": {"workload": W["name"], "slices_per_pass": K,
                   "len_storage": args.len_storage, "index": "4-bit delta",
                   "gather_operands": "f16 (tile, factor-1)" if args.half else "f32",
                   "forward": "tile-staged (64x64 shared-memory tiles)" if args.tiles
                              else "ray-ordered",
                   "step": f"one PML iteration over all {S} slices",
                   "l2": "inputs larger than L2 (system matrix "
                         f"{(info['forward_bytes'] + info['backward_bytes']) / 1e9:.1f} GB "
                         "streamed per step)",
                   "parallelism": f"replicas x{ws}"},
        "roofline": roofline, "clocks": clk.summary(), "gpu_launches": launches,
        "setup_ms": info["setup_ms"], "num_segments_per_slice": info["num_segments"],
        "device_bytes": info["device_bytes"],
        "rel_l2_vs_fp64": rel, "plain_fp32": plain, "e2e": e2e, "autotune": tuned,
        "cpu_baseline": cpu,
        "wall_s": time.time() - t0,
    }
    print(json.dumps(line), flush=True)


def fp64_check(args, W, theta, sino, prm, tg, torch, dev):
    """Per-iteration relative L2 against the GPU FP64 mode on a slice subset,
    over the workload's full iteration count, for the mixed path (its
    arithmetic per slice does not depend on the slices per pass) and the
    plain FP32 path (the reference's operation order)."""
    import numpy as np
    n = W["fp64_slices"]
    sub = sino[:, :n, :].contiguous()
    configs = {
        "fp64": dict(len_storage="f32", mode="fp64"),
        "mixed": dict(len_storage=args.len_storage, mode="fast", delta_index=True,
                      forward_tiles=args.tiles, backward_staged=args.staged,
                      half_gathers=args.half),
        "plain_fp32": dict(len_storage="f32", mode="exact"),
    }
    runs = {}
    for key, kw in configs.items():
        p = tg.Plan(W["P"], n, W["C"], theta, **kw)
        p.set_stream(torch.cuda.current_stream().cuda_stream)
        p.set_sinogram(sub, apply_abs=True)
        p.reset_recon("pml")
        snaps = []
        for _ in range(W["iters"]):
            p.iterate("pml", 1, prm)
            snaps.append(p.get_recon("pml"))
        runs[key] = snaps
        p.close()
    out = {"slices": n, "iterations": W["iters"], "reference": "GPU FP64 mode"}
    for key in ("mixed", "plain_fp32"):
        errs = [float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b))
                for a, b in zip(runs[key], runs["fp64"])]
        out[key] = {"max": max(errs), "final": errs[-1], "per_iteration": errs}
    return out


def plain_path(args, W, theta, sino, prm, tg, torch, stream):
    n = W["plain_slices"]
    sub = sino[:, :n, :].contiguous()
    p = tg.Plan(W["P"], n, W["C"], theta, len_storage="f32", slices_per_pass=1,
                mode="exact")
    p.set_stream(stream)
    info = p.info()
    p.set_sinogram(sub, apply_abs=True)
    p.reset_recon("pml")
    for _ in range(max(1, args.warmup // 2)):
        p.iterate("pml", 1, prm)
    torch.cuda.synchronize()
    steps = max(2, args.steps // 2)
    ms = time_iterations(p, "pml", prm, steps, stream, torch)
    p.close()
    return {"value": n * steps / (ms / 1000.0), "unit": "slice-iter/s",
            "slices": n, "steps": steps, "setup_ms": info["setup_ms"],
            "matrix_bytes": info["forward_bytes"] + info["backward_bytes"],
            "config": "f32 lengths, explicit int32 indices, 1 slice per pass, "
                      "reference operation order"}


def end_to_end(args, W, theta, sino, prm, tg, torch, stream):
    """Whole reconstructions through the C ABI: plan creation (tracing),
    sinogram upload from pinned host memory, iterations, download."""
    import numpy as np
    host_sino = sino.cpu().pin_memory()
    host = host_sino.numpy()
    out = np.empty((W["S"], W["C"], W["C"]), np.float32)
    times = []
    for i in range(args.e2e_warmup + args.e2e_steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        p = tg.Plan(W["P"], W["S"], W["C"], theta, len_storage=args.len_storage,
                    slices_per_pass=args.slices_per_pass, mode="fast",
                    delta_index=True, forward_tiles=args.tiles,
                    backward_staged=args.staged, half_gathers=args.half)
        p.set_stream(stream)
        p.set_sinogram(host, apply_abs=True)
        p.reset_recon("pml")
        p.iterate("pml", W["iters"], prm)
        p.get_recon("pml", out=None)
        p.synchronize()
        dt = time.perf_counter() - t
        p.close()
        if i >= args.e2e_warmup:
            times.append(dt)
    per = statistics.median(times)
    return {"value": W["S"] * W["iters"] / per, "unit": "slice-iter/s",
            "h2d_bytes_per_step": int(host.nbytes),
            "d2h_bytes_per_step": int(out.nbytes),
            "step": f"plan creation + upload + {W['iters']} iterations + download",
            "seconds_per_step": per, "steps": len(times)}


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
    ap.add_argument("--autotune", action="store_true",
                    help="time the plan configurations on a 16-slice sample first "
                         "and run the fastest")
    ap.add_argument("--no-plain", dest="plain", action="store_false")
    ap.add_argument("--no-e2e", dest="e2e", action="store_false")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-fp64-check", dest="fp64_check", action="store_false")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--e2e-warmup", type=int, default=1)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("note: fewer than 3 warm-up steps", file=sys.stderr)
    W = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, W)
    else:
        run_ours(args, W)


if __name__ == "__main__":
    main()
