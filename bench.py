#!/usr/bin/env python
"""Benchmark of the GB300 volume hot path on the sort-last workload.

Workload (one frame = one step): a 512^3 fp32 field of 64 seeded Gaussian
blobs, split by chopSuey into 2x2x2 bricks (8 bricks with a one-voxel upper
ghost layer, 540 MB resident in HBM), rendered as 8 virtual ranks at
1024x1024 with 256 seeded orbit cameras; every rank marches its brick and the
rank images are blended front to back in fp32.  Step 0.5 voxel, early
termination at alpha 0.99, 256-entry ramp transfer function.

Prints one JSON line (rank 0).  `value` = Gsamples/s (march loop-body
executions per second) with everything resident in HBM; `e2e` = the same
metric through the public C ABI with a pinned host frame buffer (camera in,
frame out every step).  `--impl reference` times the CPU restatement of the
reference path (the reference's own build cannot be compiled here) on the
host cores instead.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gsamples/s & ms/frame (fwd; fwd+adjoint) 512³ DVR @1024² on 1 GB300 vs plain"
WORKLOAD = ("sort-last DVR: {n}^3 fp32 64-blob field, chopSuey 2x2x2 (8 bricks, 8 virtual ranks), "
            "{size}x{size}, {cams} orbit cameras, dt 0.5, ET 0.99, fp32 ordered-over composite")
DEVVIEW_BYTES = 80


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=256)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["aloha", "reference"], default="aloha")
    ap.add_argument("--n", type=int, default=512, help="volume edge (voxels)")
    ap.add_argument("--size", type=int, default=1024, help="image edge (pixels)")
    ap.add_argument("--cameras", type=int, default=256)
    ap.add_argument("--batch-views", type=int, default=64)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU work of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-large", action="store_true",
                    help="skip the 1024^3 / 64-brick / 2048^2 section (about 110 GB of device memory)")
    ap.add_argument("--adjoint-case", choices=["small", "volume"], default="small",
                    help="with --only-adjoint: the 128^3 single-brick case, or the bench volume (--n, --size) "
                         "in 8 bricks as one rank over 2 cameras")
    ap.add_argument("--adjoint-k", type=int, default=32, help="checkpoint every K samples in the adjoint sections")
    ap.add_argument("--only-adjoint", action="store_true",
                    help="run only the 128^3, 16 x 256^2 forward + adjoint configuration and print its timings")
    ap.add_argument("--only-batched", action="store_true",
                    help="run only the uneven batched configuration (--n volume, --batch-big views at 1024^2 and "
                         "--batch-small at 512^2) and print its timings")
    ap.add_argument("--batch-big", type=int, default=64)
    ap.add_argument("--batch-small", type=int, default=32)
    ap.add_argument("--batch-staging", choices=["tune", "0", "1"], default="tune",
                    help="with --only-batched: autotune, or fix the stencil staging at the 8x4 tile")
    ap.add_argument("--profile", action="store_true", help="short run for ncu (no baselines, no clocks)")
    ap.add_argument("--reference-kind", choices=["auto", "reference", "port"], default="auto",
                    help="--impl reference: time the reference's own CPU-compiled raygen (oracle/_ref, where its "
                         "sources or build are present), the CPU restatement, or the first available")
    return ap.parse_args()


# ------------------------------------------------------------------ helpers

class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
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
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for name, val in zip(names, f[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(kernel: str):
    """dram bytes per launch from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", f"{kernel}.traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


def build_scene(args, device):
    from aloha_gb300 import scenes as S
    from aloha_gb300 import volfile as V
    n = args.n
    vol = S.blob_field((n, n, n), 64, (n / 16.0, n / 6.4), seed=2001, device=device)
    descs = V.chopsuey_split((n, n, n), 8)
    vox = [V.brick_voxels(vol, d) for d in descs]
    tf = S.ramp_tf()
    cams = S.orbit_cameras((n, n, n), args.cameras, args.size, args.size, seed=2002)
    return vol, descs, vox, tf, cams


def bricks_hit(descs, cam, W, H, stride=8):
    """Bricks whose space box any (subsampled) pixel ray enters."""
    org, d00, du, dv = (np.asarray(c, np.float64) for c in cam)
    ys, xs = np.meshgrid(np.arange(0, H, stride) + 0.5, np.arange(0, W, stride) + 0.5, indexing="ij")
    dirs = d00[None, None] + xs[..., None] * du + ys[..., None] * dv
    dirs /= np.linalg.norm(dirs, axis=-1, keepdims=True)
    dirs = np.where(np.abs(dirs) < 1e-5, 1e-5, dirs)
    hit = []
    for k, d in enumerate(descs):
        lo = (np.asarray(d["space_lo"]) - org) / dirs
        hi = (np.asarray(d["space_hi"]) - org) / dirs
        t0 = np.maximum(np.minimum(lo, hi).max(-1), 0)
        t1 = np.maximum(lo, hi).min(-1)
        if np.any(t0 < t1):
            hit.append(k)
    return hit


def algorithmic_bytes(descs, hit, n_tf, W, H):
    vox = sum(np.prod([descs[k]["voxel_hi"][a] - descs[k]["voxel_lo"][a] for a in range(3)]) for k in hit)
    return int(vox) * 4 + n_tf * 16 + W * H * 4


# --------------------------------------------------------------- CPU arms

def cpu_render_sample(descs, vox_np, tf, cams, W, H, target_s, threads=0, max_views=None):
    """Oracle (CPU restatement, OpenMP over rows) on a bounded sample of rows
    of the first views; returns (samples, seconds, rows, views, threads)."""
    from oracle import oracle as O
    O.lib()
    n_thr = threads or O.lib().ora_max_threads()
    params = O.make_params()
    scheds = {}
    total_s, total_samples, rows_done, views_used = 0.0, 0, 0, set()
    # bands of 16 rows spread over the image (one OpenMP row per thread), views
    # in order, until the time target
    band = 16
    per_view_rows = list(range(0, H, H // 8))
    for vi, cam in enumerate(cams if max_views is None else cams[:max_views]):
        c = O.make_camera(*cam)
        if vi not in scheds:
            scheds[vi] = O.schedule(descs, 8, list(c.org))
        for y in per_view_rows:
            t0 = time.perf_counter()
            r = O.render(descs, vox_np, tf, c, W, H, params, sched=scheds[vi], rows=(y, min(H, y + band)),
                         threads=n_thr, want=())
            total_s += time.perf_counter() - t0
            total_samples += r["samples"]
            rows_done += min(H, y + band) - y
            views_used.add(vi)
            if total_s >= target_s:
                return total_samples, total_s, rows_done, len(views_used), n_thr
    return total_samples, total_s, rows_done, len(views_used), n_thr


def workload_config(args, n_cams, world):
    """The config dict of the workload, shared by both arms."""
    from aloha_gb300 import volfile as V
    descs = V.chopsuey_split((args.n,) * 3, 8)
    brick_mb = algorithmic_bytes(descs, range(len(descs)), 0, 0, 0) / 1e6
    return {"workload": WORKLOAD.format(n=args.n, size=args.size, cams=n_cams), "volume": [args.n] * 3,
            "bricks": 8, "virtual_ranks": 8, "image": [args.size, args.size], "cameras": n_cams,
            "parallelism": f"replicas x{world} (views)",
            "l2": f"inputs {'larger' if brick_mb > 129 else 'smaller'} than L2 ({brick_mb:.0f} MB of bricks per view)",
            "seeds": {"volume": 2001, "cameras": 2002}}


def reference_kind(requested: str) -> str:
    """"reference": the reference's own deviceCode.cpp raygen and Partitioner,
    compiled on the CPU from its sources (oracle/_ref), usable wherever those
    sources are present or that build exists for this machine; "port": the
    CPU restatement (oracle/), which runs everywhere."""
    if requested == "port":
        return "port"
    try:
        from oracle import reference as R
        ok = R.loadable()
    except Exception:
        ok = False
    if requested == "reference" and not ok:
        raise SystemExit("--reference-kind reference: the reference build is not available here")
    return "reference" if ok else "port"


def reference_arm(args):
    """--impl reference: the reference path on all host cores, rank 0 only.
    The reference's OptiX/MPI/IceT build cannot run here; its own CPU-compiled
    raygen and Partitioner (oracle/_ref) are timed where available, else the
    CPU restatement."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from aloha_gb300 import scenes as S
    from aloha_gb300 import volfile as V
    from oracle import oracle as O
    n, W = args.n, args.size
    vol = S.blob_field((n, n, n), 64, (n / 16.0, n / 6.4), seed=2001)
    descs = V.chopsuey_split((n, n, n), 8)
    vox = [V.brick_voxels(vol, d) for d in descs]
    tf = S.ramp_tf()
    cams = S.orbit_cameras((n, n, n), args.cameras, W, W, seed=2002)
    threads = O.lib().ora_max_threads()
    params = O.make_params()
    rows_per_step = 16
    kind = reference_kind(args.reference_kind)
    if kind == "reference":
        from oracle import reference as R
        band = R.BandRenderer(descs, vox, tf, W, W, 8, dt=params.dt, jitter_mode=params.jitter_mode,
                              threads=threads)

    # step k: band k % 8 of view k // 8, 16 rows starting at a multiple of
    # H/8 (the bands the GPU arm's cpu_baseline samples)
    def step(k):
        cam = O.make_camera(*cams[(k // 8) % len(cams)])
        y0 = (k % 8) * (W // 8)
        rows = (y0, min(W, y0 + rows_per_step))
        if kind == "reference":
            return band.render(cam, rows)[1]
        sch = O.schedule(descs, 8, list(cam.org))
        r = O.render(descs, vox, tf, cam, W, W, params, sched=sch, rows=rows, threads=threads, want=())
        return r["samples"]

    for k in range(args.warmup):
        step(k)
    t0 = time.perf_counter()
    samples = 0
    for k in range(args.steps):
        samples += step(args.warmup + k)
    dt = time.perf_counter() - t0
    g = samples / dt / 1e9
    line = {"metric": METRIC, "value": g, "unit": "Gsamples/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": workload_config(args, len(cams), args.gpus),
            "step": "one 16-row band of one view (8 bands per view, every H/8 rows)",
            "cpu_baseline": {"value": g, "unit": "Gsamples/s", "cores": threads, "kind": kind,
                             "sample": f"{args.steps} steps x {rows_per_step} rows x {W} pixels"},
            "e2e": {"value": g, "unit": "Gsamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU arm

def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
        return
    import torch
    import torch.distributed as dist

    from aloha_gb300 import abi
    from aloha_gb300.replicas import max_over_ranks, shard_views, sum_over_ranks

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.only_batched:
        from aloha_gb300 import scenes as S
        n = args.n
        vol = S.blob_field((n, n, n), 64, (n / 16.0, n / 6.4), seed=2001, device=dev)
        staging = None if args.batch_staging == "tune" else int(args.batch_staging)
        print(json.dumps(uneven_batched_section(vol, dev, args.batch_big, args.batch_small, staging=staging,
                                                profile=args.profile)), flush=True)
        return
    if args.only_adjoint:
        from aloha_gb300 import scenes as S
        if args.adjoint_case == "volume":
            vol, descs, _, _, cams = build_scene(args, dev)
            res = adjoint_section(f"{args.n}^3 @{args.size}^2, 8 bricks as 1 rank", vol, descs, cams[:2], args.size,
                                  args.size, args.adjoint_k, torch.cuda.current_stream(), dev)
        else:
            v4 = S.blob_field((128, 128, 128), 16, (4.0, 12.0), seed=4001, device=dev)
            c4 = S.orbit_cameras((128, 128, 128), 16, 256, 256, seed=4002)
            res = adjoint_section("128^3 single brick, 16 x 256^2", v4, S.single_brick((128, 128, 128)), c4, 256,
                                  256, args.adjoint_k, torch.cuda.current_stream(), dev)
        print(json.dumps(res), flush=True)
        return

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    vol, descs, vox, tf, cams = build_scene(args, dev)
    W = H = args.size
    ctx = abi.Context(local)
    ctx.set_bricks(descs, vox)
    ctx.set_transfer_function(tf)
    ctx.set_ranks(8)
    ctx.set_params()
    # replicas only: rank r renders cameras r, r+N, ...
    mine = shard_views(len(cams), rank, world)
    stream = torch.cuda.Stream(device=dev)
    fb = torch.zeros((H, W), dtype=torch.int32, device=dev)

    # per-camera sample counts and algorithmic bytes (untimed)
    samples_of, bytes_of = {}, {}
    with torch.cuda.stream(stream):
        for ci in mine:
            ctx.set_camera(0, *cams[ci])
            ctx.resize(0, W, H)
            ctx.render(0, fb, stream)
            samples_of[ci] = ctx.stats().samples
            bytes_of[ci] = algorithmic_bytes(descs, bricks_hit(descs, cams[ci], W, H), tf.shape[0], W, H)

    # work-division sweep of the single-view render (untimed): the pixel split
    # at three chunk shapes, and the (chunk, rank) split
    none, staged = abi.STAGING_NONE, abi.STAGING_NEXT_SAMPLE
    # (split, chunk w, h, chunk order, staging, lane-group share per mille)
    schedules = {"pixels 8x4": (abi.SPLIT_PIXELS, 8, 4, abi.CHUNKS_PROBED, none, 0),
                 "pixels 8x4 lane groups 1%": (abi.SPLIT_PIXELS, 8, 4, abi.CHUNKS_PROBED, none, 10),
                 "pixels 8x4 lane groups 4%": (abi.SPLIT_PIXELS, 8, 4, abi.CHUNKS_PROBED, none, 40),
                 "pixels 8x4 lane groups 15%": (abi.SPLIT_PIXELS, 8, 4, abi.CHUNKS_PROBED, none, 150),
                 "pixels 8x4 staged": (abi.SPLIT_PIXELS, 8, 4, abi.CHUNKS_PROBED, staged, 0),
                 "pixels 8x4 ring order": (abi.SPLIT_PIXELS, 8, 4, abi.CHUNKS_RING, none, 0),
                 "pixels 8x8": (abi.SPLIT_PIXELS, 8, 8, abi.CHUNKS_PROBED, none, 0),
                 "pixels 16x8": (abi.SPLIT_PIXELS, 16, 8, abi.CHUNKS_PROBED, none, 0),
                 "ranks": (abi.SPLIT_RANKS, 0, 0, abi.CHUNKS_AUTO, none, 0)}
    sched_ms = {}
    for name, (split, tw, th, chunks, stage, lg) in schedules.items():
        ctx.set_render_split(split)
        ctx.set_render_tile(tw, th)
        ctx.set_chunk_order(chunks)
        ctx.set_render_staging(stage)
        ctx.set_lane_groups(lg)
        probe = mine[:8]
        for ci in probe[:2]:
            ctx.set_camera(0, *cams[ci])
            ctx.render(0, fb, stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ms = 0.0
        for ci in probe:
            ctx.set_camera(0, *cams[ci])
            e0.record(stream)
            ctx.render(0, fb, stream)
            e1.record(stream)
            e1.synchronize()
            ms += e0.elapsed_time(e1)
        sched_ms[name] = ms / len(probe)
    best = min(sched_ms, key=sched_ms.get)
    split, tw, th, chunks, stage, lg = schedules[best]
    ctx.set_render_split(split)
    ctx.set_render_tile(tw, th)
    ctx.set_chunk_order(chunks)
    ctx.set_render_staging(stage)
    ctx.set_lane_groups(lg)
    kernel = ("render_split_kernel" if split == abi.SPLIT_RANKS else
              f"render_warps_kernel<{tw},{th},5,{stage}{',4' if lg else ''}>")
    # our kernels per frame: the render, plus the chunk probe (which also
    # counts the classes), scan and scatter of the cost order, and for the
    # rank split its mask, three scan kernels and emit
    probed = chunks == abi.CHUNKS_PROBED or (chunks == abi.CHUNKS_AUTO and W * H >= 512 * 512)
    launches_per_frame = (6 if split == abi.SPLIT_RANKS else 1) + (3 if probed else 0)

    steps = [mine[k % len(mine)] for k in range(args.steps)]
    for k in range(args.warmup):
        ctx.set_camera(0, *cams[mine[k % len(mine)]])
        ctx.render(0, fb, stream)
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in steps]
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        t_start.record(stream)
        for (e0, e1), ci in zip(ev, steps):
            ctx.set_camera(0, *cams[ci])
            e0.record(stream)
            ctx.render(0, fb, stream)
            e1.record(stream)
        t_end.record(stream)
        barrier()
    elapsed_ms = t_start.elapsed_time(t_end)
    launch_ms = [e0.elapsed_time(e1) for e0, e1 in ev]
    total_samples = sum(samples_of[ci] for ci in steps)
    elapsed_ms = max_over_ranks(elapsed_ms, dev)
    total_samples = int(sum_over_ranks(total_samples, dev))
    value = total_samples / (elapsed_ms * 1e-3) / 1e9

    # roofline of the fused render kernel: algorithmic bytes / launch duration
    mean_bytes = float(np.mean([bytes_of[ci] for ci in steps]))
    mean_launch = float(np.mean(launch_ms))
    peak, peak_kind = measured_peaks()
    achieved = mean_bytes / (mean_launch * 1e-3) / 1e9
    # the committed capture describes the default workload only
    default_workload = args.n == 512 and args.size == 1024
    traffic = profile_traffic(kernel.split("<")[0]) if default_workload else None

    result = {"metric": METRIC, "value": value, "unit": "Gsamples/s", "n_gpus": world, "steps": args.steps,
              "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
              "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
              "config": workload_config(args, len(cams), world),
              "ms_per_frame": elapsed_ms / args.steps,
              "samples_per_frame": total_samples / max(1, args.steps * world),
              "gpu_launches": args.steps * launches_per_frame,
              "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                           "frac": achieved / peak, "peak_kind": peak_kind,
                           "traffic": traffic["bytes_per_launch"] if traffic else None,
                           "kernel": kernel, "schedule": best, "schedule_sweep_ms": sched_ms,
                           "algorithmic_bytes_per_launch": mean_bytes, "launch_ms": mean_launch}}
    # nvidia-smi samples every 100 ms: a timed region shorter than that may hold none
    result["clocks"] = clk.summary() or {"sm_mhz": None, "sm_max_mhz": None, "samples": 0, "reasons": [],
                                         "note": "no clock sample fell inside the timed region"}

    if not args.profile:
        # e2e: through the C ABI with a pinned host frame buffer every step
        fb_host = torch.zeros((H, W), dtype=torch.int32).pin_memory()
        for k in range(args.warmup):
            ctx.set_camera(0, *cams[mine[k % len(mine)]])
            ctx.render(0, fb_host, stream)
        barrier()
        t0 = time.perf_counter()
        for ci in steps:
            ctx.set_camera(0, *cams[ci])
            ctx.render(0, fb_host, stream)
        barrier()
        e2e_s = time.perf_counter() - t0
        e2e_s = max_over_ranks(e2e_s, dev)
        sched_bytes = 4 * (2 * 8 + 1 + 8)
        result["e2e"] = {"value": total_samples / e2e_s / 1e9, "unit": "Gsamples/s",
                         "ms_per_frame": e2e_s / args.steps * 1e3,
                         "h2d_bytes_per_step": DEVVIEW_BYTES + sched_bytes, "d2h_bytes_per_step": W * H * 4}

        if not args.no_batched and rank == 0:
            result["batched"] = batched_section(ctx, cams, mine, W, H, args, stream, dev, samples_of)
            result["batched_uneven"] = uneven_batched_section(vol, dev)

        if not args.no_adjoint and rank == 0:
            from aloha_gb300 import scenes as S
            # the headline volume and image as one virtual rank
            adj = [adjoint_section("512^3 @1024^2, 8 bricks as 1 rank", vol, descs, cams[:4], W, H, args.adjoint_k,
                                   stream, dev)]
            # the differentiable configuration: 128^3 single brick, 16 views at 256^2
            v4 = S.blob_field((128, 128, 128), 16, (4.0, 12.0), seed=4001, device=dev)
            c4 = S.orbit_cameras((128, 128, 128), 16, 256, 256, seed=4002)
            adj.append(adjoint_section("128^3 single brick, 16 x 256^2", v4, S.single_brick((128, 128, 128)), c4,
                                       256, 256, args.adjoint_k, stream, dev))
            result["adjoint"] = adj
            result["autograd"] = autograd_section(dev)

        if not args.no_cpu_baseline and rank == 0:
            vol_np = vol.cpu().numpy()
            from aloha_gb300 import volfile as V
            vox_np = [V.brick_voxels(vol_np, d) for d in descs]
            s, sec, rows, nv, thr = cpu_render_sample(descs, vox_np, tf, cams, W, H, args.cpu_seconds)
            result["cpu_baseline"] = {"value": s / sec / 1e9, "unit": "Gsamples/s", "cores": thr, "kind": "port",
                                      "sample": f"{rows} rows (16-row bands, 8 per view) of {nv} view(s) at {W} px, "
                                                f"{s} samples in {sec:.1f} s"}
        if not args.no_large and rank == 0:
            ctx.close()
            torch.cuda.empty_cache()
            result["large"] = large_section(dev)
    if rank == 0:
        print(json.dumps(result), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


def adjoint_section(name, vol, descs, cams, W, H, k, stream, dev):
    """Forward (checkpoints every k samples) and adjoint of an L2 image loss
    over `cams` views of one virtual rank; times both with CUDA events."""
    import torch

    from aloha_gb300 import abi
    from aloha_gb300 import scenes as S
    from aloha_gb300 import volfile as V
    ctx = abi.Context(dev.index or 0)
    vox = [V.brick_voxels(vol, d) for d in descs]
    ctx.set_bricks(descs, vox)
    ctx.set_ranks(1)
    ctx.set_params()
    n = vol.shape[0]
    for v, cam in enumerate(cams):
        ctx.set_camera(v, *cam)
        ctx.resize(v, W, H)
    nv = len(cams)
    target = torch.empty((nv, H, W, 4), dtype=torch.float32, device=dev)
    ctx.set_transfer_function(S.seeded_tf(77))
    for v in range(nv):
        ctx.forward(v, target[v], k, stream)
    ctx.set_transfer_function(S.ramp_tf())
    img = torch.empty_like(target)
    dtf = torch.zeros((256, 4), dtype=torch.float32, device=dev)
    dden = torch.zeros(tuple(vol.shape), dtype=torch.float32, device=dev)

    def fwd(batched=False):
        if batched:  # all views in one aloha_forward_views launch
            ctx.forward_views(list(range(nv)), [img[v] for v in range(nv)], k, stream)
            return
        for v in range(nv):
            ctx.forward(v, img[v], k, stream)

    def bwd(grad, with_tf=True, with_density=True, summed=False):
        if summed:  # all views in one aloha_backward_views call
            ctx.backward_views(list(range(nv)), [grad[v] for v in range(nv)], dtf if with_tf else None,
                               dden if with_density else None, (0, 0, 0) if with_density else None,
                               (n, n, n) if with_density else None, stream)
            return
        for v in range(nv):
            if with_density:
                ctx.backward(v, grad[v], dtf if with_tf else None, dden, (0, 0, 0), (n, n, n), stream)
            else:
                ctx.backward(v, grad[v], dtf, None, None, None, stream)

    fwd()
    grad = (2.0 * (img - target)).contiguous()
    bwd(grad)
    torch.cuda.synchronize()
    samples = 0
    for v in range(nv):
        ctx.forward(v, img[v], k, stream)
        samples += ctx.stats().samples
    reps = 3
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fwd_ms, bwd_ms = 0.0, 0.0
    for _ in range(reps):
        torch.cuda.synchronize()
        e[0].record(stream)
        fwd()
        e[1].record(stream)
        bwd(grad)
        e[2].record(stream)
        torch.cuda.synchronize()
        fwd_ms += e[0].elapsed_time(e[1]) / reps
        bwd_ms += e[1].elapsed_time(e[2]) / reps
    # density gradient only (the backward skips empty space)
    den_ms = 0.0
    for _ in range(reps):
        torch.cuda.synchronize()
        e[0].record(stream)
        fwd()
        e[1].record(stream)
        bwd(grad, with_tf=False)
        e[2].record(stream)
        torch.cuda.synchronize()
        den_ms += e[1].elapsed_time(e[2]) / reps
    # transfer-function gradient only (no shading or stencil adjoint)
    tf_ms = 0.0
    for _ in range(reps):
        torch.cuda.synchronize()
        e[0].record(stream)
        fwd()
        e[1].record(stream)
        bwd(grad, with_density=False)
        e[2].record(stream)
        torch.cuda.synchronize()
        tf_ms += e[1].elapsed_time(e[2]) / reps
    # the views in one launch each way: aloha_forward_views, then their
    # gradients summed by one aloha_backward_views call (one accumulation
    # buffer cleared and folded once, one host wait, one launch)
    sum_ms, sum_den_ms, fwdv_ms = 0.0, 0.0, 0.0
    for _ in range(reps):
        for with_tf in (True, False):
            torch.cuda.synchronize()
            e[0].record(stream)
            fwd(batched=True)
            e[1].record(stream)
            bwd(grad, with_tf=with_tf, summed=True)
            e[2].record(stream)
            torch.cuda.synchronize()
            fwdv_ms += e[0].elapsed_time(e[1]) / (2 * reps)
            if with_tf:
                sum_ms += e[1].elapsed_time(e[2]) / reps
            else:
                sum_den_ms += e[1].elapsed_time(e[2]) / reps
    ctx.close()
    return {"config": name, "views": nv, "image": [W, H], "checkpoint_every": k,
            "fwd_ms_per_view": fwd_ms / nv, "adjoint_ms_per_view": bwd_ms / nv,
            "fwd_plus_adjoint_over_fwd": (fwd_ms + bwd_ms) / fwd_ms,
            "adjoint_density_only_ms_per_view": den_ms / nv,
            "fwd_plus_density_adjoint_over_fwd": (fwd_ms + den_ms) / fwd_ms,
            "adjoint_tf_only_ms_per_view": tf_ms / nv,
            "fwd_plus_tf_adjoint_over_fwd": (fwd_ms + tf_ms) / fwd_ms,
            "fwd_views_ms_per_view": fwdv_ms / nv,
            "adjoint_views_summed_ms_per_view": sum_ms / nv,
            "adjoint_views_summed_density_only_ms_per_view": sum_den_ms / nv,
            "views_fwd_plus_adjoint_over_fwd": (fwdv_ms + sum_ms) / fwdv_ms,
            "samples_per_view": samples / nv,
            "fwd_gsamples_per_s": samples / (fwd_ms * 1e-3) / 1e9,
            "fwd_plus_adjoint_gsamples_per_s": samples / ((fwd_ms + bwd_ms) * 1e-3) / 1e9}


def autograd_section(dev, steps=5):
    """The differentiable configuration through the torch binding, the call a
    training loop makes: render_views of 16 views (one forward launch), an L2
    loss against targets of a second transfer function, loss.backward() for
    the transfer-function and density gradients (one summed backward).  CUDA
    events around whole steps."""
    import torch

    from aloha_gb300 import scenes as S
    from aloha_gb300.autograd import DifferentiableRenderer, render_views
    dims = (128, 128, 128)
    den = S.blob_field(dims, 16, (4.0, 12.0), seed=4001, device=dev).contiguous().requires_grad_(True)
    cams = S.orbit_cameras(dims, 16, 256, 256, seed=4002)
    r = DifferentiableRenderer(dims, bricks=1, checkpoint_every=32)
    for v, cam in enumerate(cams):
        r.set_camera(v, cam, 256, 256)
    views = list(range(16))
    with torch.no_grad():
        target = render_views(r, torch.from_numpy(S.seeded_tf(77)).to(dev), den.detach(), views, (256, 256))
    tf = torch.from_numpy(S.ramp_tf()).to(dev).requires_grad_(True)

    def step():
        tf.grad = None
        den.grad = None
        loss = ((render_views(r, tf, den, views, (256, 256)) - target) ** 2).sum()
        loss.backward()

    for _ in range(3):
        step()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    r.close()
    return {"config": "128^3 single brick, 16 x 256^2, torch.autograd (render_views, L2 loss, both gradients)",
            "ms_per_step": ms, "ms_per_view": ms / 16}


def batched_section(ctx, cams, mine, W, H, args, stream, dev, samples_of):
    """64 views in one persistent launch (CUDA graph) vs 64 plain launches."""
    import torch
    nv = min(args.batch_views, len(mine))
    views = list(range(1, nv + 1))
    for v, ci in zip(views, mine[:nv]):
        ctx.set_camera(v, *cams[ci])
        ctx.resize(v, W, H)
    fbs = [torch.zeros((H, W), dtype=torch.int32, device=dev) for _ in views]
    b = ctx.batch(views, fbs)
    tw, th, _ = b.autotune(stream, reps=1)

    def timed(fn, reps=3):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    stage, steps = b.staging(), b.unroll()
    by_stage = staging_sweep(b, stream, timed)
    ms_graph = timed(lambda: b.launch_graph(stream))

    def plain():
        for v, f in zip(views, fbs):
            ctx.render(v, f, stream)

    ms_plain = timed(plain)
    samples = sum(samples_of[ci] for ci in mine[:nv])
    b.close()
    return {"views": nv, "tile": [tw, th], "staging": STAGING_NAMES[stage], "unroll": steps,
            "ms_batch_by_staging": by_stage, "ms_batch": ms_graph, "ms_plain_launches": ms_plain,
            "speedup_vs_plain": ms_plain / ms_graph, "gsamples_per_s": samples / (ms_graph * 1e-3) / 1e9}


STAGING_NAMES = {0: "none", 1: "next sample (cp.async, shared memory)"}


def staging_sweep(b, stream, timed):
    """Graph-launch time of the batch at its tuned tile with each staging, and
    with direct loads two march steps per loop trip (untimed for the
    headline); leaves the tuned staging and unroll set."""
    chosen, steps = b.staging(), b.unroll()
    out = {}
    b.set_unroll(1)
    for stage, name in STAGING_NAMES.items():
        b.set_staging(stage)
        out[name] = timed(lambda: b.launch_graph(stream))
    b.set_staging(0)
    b.set_unroll(2)
    out["none, two steps per loop trip"] = timed(lambda: b.launch_graph(stream))
    b.set_staging(chosen)
    b.set_unroll(steps)
    return out


def uneven_batched_section(vol, dev, big=64, small=32, staging=None, profile=False):
    """The batched configuration: the same 512^3 field in uneven 3x2x2 bricks
    (x cuts 200, 380; y 256; z 300), 64 views at 1024^2 and 32 at 512^2 in one
    graph-captured persistent launch (autotuned), against the same views as
    plain aloha_render launches.  `staging` fixes the stencil staging at the
    8x4 tile instead of autotuning; `profile` launches the batch once and
    times nothing (for ncu)."""
    import torch

    from aloha_gb300 import abi
    from aloha_gb300 import scenes as S
    from aloha_gb300 import volfile as V
    n = vol.shape[0]
    descs = S.grid_split((n, n, n), ([n * 200 // 512, n * 380 // 512], [n // 2], [n * 300 // 512]))
    ctx = abi.Context(dev.index or 0)
    ctx.set_bricks(descs, [V.brick_voxels(vol, d) for d in descs])
    ctx.set_transfer_function(S.ramp_tf())
    ctx.set_ranks(len(descs))
    ctx.set_params()
    sizes = [1024] * big + [512] * small
    cams = [S.orbit_cameras((n, n, n), 1, w, w, seed=3002 + i)[0] for i, w in enumerate(sizes)]
    stream = torch.cuda.current_stream()
    fbs = []
    samples = 0
    for v, (w, cam) in enumerate(zip(sizes, cams)):
        ctx.set_camera(v, *cam)
        ctx.resize(v, w, w)
        fbs.append(torch.zeros((w, w), dtype=torch.int32, device=dev))
        ctx.render(v, fbs[-1], stream)
        samples += ctx.stats().samples
    b = ctx.batch(list(range(len(sizes))), fbs)
    if staging is None:
        tw, th, _ = b.autotune(stream, reps=1)
    else:
        tw, th = 8, 4
        b.set_staging(staging)
        b.set_config(tw, th)
    if profile:
        b.launch_graph(stream)
        torch.cuda.synchronize()
        chosen = b.staging()
        b.close()
        ctx.close()
        return {"config": f"{n}^3 in {len(descs)} uneven bricks, {big} views at 1024^2 + {small} at 512^2",
                "tile": [tw, th], "staging": STAGING_NAMES[chosen], "profile": True}

    def timed(fn, reps=3):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    stage, steps = b.staging(), b.unroll()
    by_stage = staging_sweep(b, stream, timed)
    ms_batch = timed(lambda: b.launch_graph(stream))
    ms_plain = timed(lambda: [ctx.render(v, f, stream) for v, f in enumerate(fbs)])
    b.close()
    ctx.close()
    px = sum(w * w for w in sizes)
    return {"config": f"{n}^3 in {len(descs)} uneven bricks, {big} views at 1024^2 + {small} at 512^2",
            "tile": [tw, th], "staging": STAGING_NAMES[stage], "unroll": steps, "ms_batch_by_staging": by_stage,
            "ms_batch": ms_batch, "ms_plain_launches": ms_plain,
            "speedup_vs_plain": ms_plain / ms_batch, "gsamples_per_s": samples / (ms_batch * 1e-3) / 1e9,
            "ms_per_megapixel": ms_batch / (px / 2**20)}


def large_section(dev, n=1024, size=2048, views=8, k=64):
    """The large configuration: 1024^3 fp32 blobs in 4x4x4 bricks, 8 views at
    2048^2.  Render with 64 virtual ranks (both work divisions, plain and
    batched), then forward plus adjoint (TF and density) over the 8 views as
    one virtual rank with a checkpoint every 64 samples."""
    import torch

    from aloha_gb300 import abi
    from aloha_gb300 import scenes as S
    from aloha_gb300 import volfile as V
    dims = (n, n, n)
    stream = torch.cuda.current_stream()
    vol = S.blob_field(dims, 64, (n / 16.0, n / 6.4), seed=5001, device=dev)
    descs = V.chopsuey_split(dims, 64)
    ctx = abi.Context(dev.index or 0)
    ctx.set_bricks(descs, [V.brick_voxels(vol, d) for d in descs])
    del vol
    torch.cuda.empty_cache()
    ctx.set_transfer_function(S.ramp_tf())
    ctx.set_ranks(len(descs))
    ctx.set_params()
    cams = S.orbit_cameras(dims, views, size, size, seed=5004)
    for v, cam in enumerate(cams):
        ctx.set_camera(v, *cam)
        ctx.resize(v, size, size)
    fbs = [torch.zeros((size, size), dtype=torch.int32, device=dev) for _ in cams]

    def timed(fn, reps=2):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    samples = 0
    for v in range(views):
        ctx.render(v, fbs[v], stream)
        samples += ctx.stats().samples
    out = {"config": f"{n}^3 fp32 in {len(descs)} bricks ({len(descs)} virtual ranks), {views} views at {size}^2",
           "samples_per_view": samples / views}
    for name, split in (("pixels", abi.SPLIT_PIXELS), ("ranks", abi.SPLIT_RANKS)):
        ctx.set_render_split(split)
        ms = timed(lambda: [ctx.render(v, fbs[v], stream) for v in range(views)]) / views
        out[f"render_{name}_ms_per_view"] = ms
        out[f"render_{name}_gsamples_per_s"] = samples / views / (ms * 1e-3) / 1e9
    ctx.set_render_split(abi.SPLIT_AUTO)
    b = ctx.batch(list(range(views)), fbs)
    b.autotune(stream, reps=1)
    ms = timed(lambda: b.launch_graph(stream)) / views
    b.close()
    out["batched_ms_per_view"] = ms
    out["batched_gsamples_per_s"] = samples / views / (ms * 1e-3) / 1e9
    # forward + adjoint as one virtual rank
    ctx.set_ranks(1)
    img = torch.empty((views, size, size, 4), dtype=torch.float32, device=dev)
    dtf = torch.zeros((256, 4), dtype=torch.float32, device=dev)
    dden = torch.zeros(dims, dtype=torch.float32, device=dev)
    g = torch.Generator(device=dev).manual_seed(5005)
    dl = (torch.rand((size, size, 4), generator=g, device=dev) * 2.0 - 1.0).contiguous()

    def fwd():
        for v in range(views):
            ctx.forward(v, img[v], k, stream)

    def bwd(with_tf=True):
        for v in range(views):
            ctx.backward(v, dl, dtf if with_tf else None, dden, (0, 0, 0), dims, stream)

    fwd_ms = timed(fwd) / views
    bwd_ms = timed(bwd) / views
    den_ms = timed(lambda: bwd(False)) / views
    # the batch as the configuration states it: all views' forwards in one
    # launch, their gradients summed by one call
    vs = list(range(views))
    fwdv_ms = timed(lambda: ctx.forward_views(vs, [img[v] for v in vs], k, stream)) / views
    sumv_ms = timed(lambda: ctx.backward_views(vs, [dl] * views, dtf, dden, (0, 0, 0), dims, stream)) / views
    sumd_ms = timed(lambda: ctx.backward_views(vs, [dl] * views, None, dden, (0, 0, 0), dims, stream)) / views
    ctx.close()
    out.update({"checkpoint_every": k, "fwd_ms_per_view": fwd_ms, "adjoint_ms_per_view": bwd_ms,
                "fwd_plus_adjoint_over_fwd": (fwd_ms + bwd_ms) / fwd_ms,
                "adjoint_density_only_ms_per_view": den_ms,
                "fwd_plus_density_adjoint_over_fwd": (fwd_ms + den_ms) / fwd_ms,
                "fwd_views_ms_per_view": fwdv_ms, "adjoint_views_summed_ms_per_view": sumv_ms,
                "adjoint_views_summed_density_only_ms_per_view": sumd_ms,
                "views_fwd_plus_adjoint_over_fwd": (fwdv_ms + sumv_ms) / fwdv_ms})
    return out


if __name__ == "__main__":
    main()
