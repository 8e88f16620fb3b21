"""bench.py -- LK cells/s and frame-pair latency on one GB300, served-batched against the plain GPU form, for the
1920 x 1080 configuration: 4 levels, 16,200 cells of 16 x 8, 21 x 21 patch, <= 10 iterations, eps 0.01, forward-
backward check 0.5. Seeded synthetic frames (noise blurred at sigma 1.5, warped by a shift of up to 12 px plus a
smooth field of at most 0.5 px).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--streams B]

A step is one frame pair of each of B streams (default 8): the pyramids of their new frames and their per-cell flow,
as one batched step replayed from a CUDA graph (the batched form). `value` is cells/s over K steps with the frames in
HBM; the B streams' frames and pyramid sets (about 26 MB a stream) exceed the 129 MB L2, so no flush is needed. The
plain form beside it runs one stream, one vtg_build + vtg_cells per frame pair, with the L2 flushed before each.
`e2e` is the served request loop (vtg_serve_run) through the C ABI: pinned host frames in, cell records out, Poisson
arrivals from B 1080p streams at a saturating rate, continuous batching, 2 % of pairs followed by an appearance
search; beside it the same loop in its plain form, and a mixed-size served run at nominal frame rates for latency.
`--impl reference` times the reference's own CPU kernels (its C sources, built on this host by oracle/Makefile) on all
host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "intel-phi-visiontrack_gb300")
ORACLE = os.path.join(ROOT, "oracle")
sys.path.insert(0, PKG)

METRIC = "LK cells/s + p99 ms/frame-pair, served-batched vs plain GPU; ≤0.01px vs FP64"
W, H, LEVELS, CELL_W, CELL_H, PATCH = 1920, 1080, 4, 16, 8, 21
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one batched LK launch of 8 such streams, from an ncu
# capture of `bench.py --profile batch` (the same kernel and launch shape); a constant, not measured by this run
LK_TRAFFIC_BYTES = 177_114_880 + 8_196_864
CELLS = 16200


def max_over_ranks(ms: float, device) -> float:
    """The job's time: the slowest rank's (every rank times its own replica between the same barriers). One process:
    its own."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_cells_per_s(world: int, streams: int, cells: int, steps: int, total_ms: float) -> float:
    """Cells every rank tracked over the job's time: world replicas of `streams` streams of `cells` cells a step."""
    return world * streams * cells * steps / (total_ms / 1e3)


def workload(form: str, streams: int) -> dict:
    return {"workload": "per-cell LK flow, 1920x1080 frame pairs, 4 levels, 16,200 cells (16x8), 21x21 patch, "
                        "<=10 iters, eps 0.01, fb 0.5",
            "form": form, "streams_per_step": streams, "width": W, "height": H, "levels": LEVELS,
            "cells_per_pair": CELLS, "patch": PATCH,
            "l2": "batched: inputs larger than L2 (%d streams x ~26 MB of frames and pyramid sets); plain: L2 flushed "
                  "before every timed step (256 MiB write)" % streams}


class Clocks:
    """nvidia-smi sampled every 200 ms while the GPU work runs."""

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,power.draw")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        ok = [r for r in self.rows if len(r) >= 6 and r[0].replace(".", "").isdigit()]
        sm = [float(r[0]) for r in ok]
        mx = [float(r[1]) for r in ok if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in ok for i in range(4) if r[2 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def lk_flops(work: dict, w: int = PATCH, h: int = PATCH) -> float:
    """Algorithmic FLOPs of one LK launch from its counted work (vtg_batch_count: every template build, iteration and
    residual pass of both walks of every cell), with the reference's operation counts per patch operation
    (src/kern/lk_ref.c, FMA = 2): build 9 (W+2)(H+2) + 20 W H, iterate 14 W H, residual 12 W H."""
    build = 9 * (w + 2) * (h + 2) + 20 * w * h
    return float(work["builds"] * build + work["iterations"] * 14 * w * h + work["residuals"] * 12 * w * h)


def peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def frames_1080(n: int):
    import vtg_synth as S

    return [S.warp_pair(W, H, S.seeded_shift(2 + k, 0), 0.5, seed=2 + k)[:2] for k in range(n)]


def time_plain(vtg, torch, ctx, dev, steps: int, warmup: int, device: str):
    """The plain form: one vtg_build + vtg_cells call per frame pair, one pair at a time on one stream, taking the
    streams in turn (tracker j for stream j), so it does the batched step's work; L2 flushed before each timed pair."""
    B = len(dev)
    trackers = [vtg.Tracker(ctx, vtg.config(W, H, levels=LEVELS, cell_w=CELL_W, cell_h=CELL_H)) for _ in range(B)]
    stream = torch.cuda.Stream(device=device)
    sp = stream.cuda_stream
    dcells = torch.empty(CELLS * 24, dtype=torch.uint8, device=device)
    dlk = torch.empty(CELLS * 32, dtype=torch.uint8, device=device)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)
    torch.cuda.synchronize()
    for t, (f0, _) in zip(trackers, dev):
        t.build(0, f0.data_ptr(), where=vtg.DEVICE, stream=sp)

    def pair(k):
        j, cur = k % B, (k // B + 1) & 1
        f0, f1 = dev[j]
        trackers[j].build(cur, (f1 if cur else f0).data_ptr(), where=vtg.DEVICE, stream=sp)
        trackers[j].cells_device(cur ^ 1, cur, dcells.data_ptr(), dlk.data_ptr(), stream=sp)

    w = warmup * B
    for k in range(w):
        pair(k)
    steps = -(-steps // B) * B
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 255)
            ev[k][0].record(stream)
        pair(w + k)
        with torch.cuda.stream(stream):
            ev[k][1].record(stream)
    torch.cuda.synchronize()
    ms = np.array([a.elapsed_time(b) for a, b in ev])
    for t in trackers:
        t.close()
    return {"value": CELLS * steps / (ms.sum() / 1e3), "unit": "cells/s", "ms_per_pair": float(ms.mean()),
            "p50_ms_per_pair": float(np.percentile(ms, 50)), "p99_ms_per_pair": float(np.percentile(ms, 99)),
            "pairs": steps, "streams": B,
            # one pyramid launch for each level above 0, then the LK launch
            "gpu_launches_per_pair": (LEVELS - 1) + 1}


def time_batched_mix(vtg, torch, ctx, device: str, nstreams: int = 64, steps: int = 300, warmup: int = 3) -> dict:
    """Many uneven streams in one step: nstreams streams with sizes drawn uniformly (seeded) from 640x480, 1280x720 and
    1920x1080 (1,200 cells on a 16-px grid at 640x480 with 3 levels; 7,200 and 16,200 cells on 16x8 with 4 levels),
    each with its own seeded shift of up to 12 px. Every stream's pyramid sets and cell state stay on the device for
    `steps` frames, replayed from the two captured graphs; the autotuned launch shape against the default one."""
    import concurrent.futures as cf

    import vtg_synth as S

    sizes = [(640, 480), (1280, 720), (1920, 1080)]
    pick = np.random.default_rng(4).integers(0, 3, nstreams)
    with cf.ThreadPoolExecutor(min(16, os.cpu_count() or 4)) as ex:
        pairs = list(ex.map(lambda k: S.warp_pair(*sizes[pick[k]], S.seeded_shift(100 + k, 0), 0.5,
                                                  seed=100 + k)[:2], range(nstreams)))
    dev = [(torch.from_numpy(f0).to(device), torch.from_numpy(f1).to(device)) for f0, f1 in pairs]
    torch.cuda.synchronize()
    trackers = []
    for k in range(nstreams):
        w, h = sizes[pick[k]]
        small = w == 640
        trackers.append(vtg.Tracker(ctx, vtg.config(w, h, levels=3 if small else 4, cell_w=16,
                                                    cell_h=16 if small else 8)))
    batch = vtg.Batch(ctx, nstreams)
    batch.prepare(0, trackers, [d0.data_ptr() for d0, _ in dev], [0] * nstreams)
    batch.prepare(1, trackers, [d1.data_ptr() for _, d1 in dev], [1] * nstreams)
    batch.launch(0)
    batch.launch(1)
    ctx.sync()
    cells = batch.cells(1)
    default_tune = batch.get_tune()
    tuned, tuned_ms, default_ms = batch.autotune(1, reps=5)
    batch.capture(0)
    batch.capture(1)
    bstream = torch.cuda.ExternalStream(batch.stream)
    for k in range(warmup):
        batch.replay(k & 1)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for k in range(steps):
        ev[k][0].record(bstream)
        batch.replay((warmup + k) & 1)
        ev[k][1].record(bstream)
    torch.cuda.synchronize()
    ms = np.array([a.elapsed_time(b) for a, b in ev])
    batch.close()
    # the plain form on the same streams: one vtg_build + vtg_cells per frame pair, the streams in turn, one stream
    pstream = torch.cuda.Stream(device=device)
    sp = pstream.cuda_stream
    dc = torch.empty(16200 * 24, dtype=torch.uint8, device=device)
    rounds = 6
    for r in range(rounds + 1):
        if r == 1:
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(pstream)
        for k, t in enumerate(trackers):
            cur = (r + 1) & 1
            t.build(cur, dev[k][cur].data_ptr(), where=vtg.DEVICE, stream=sp)
            t.cells_device(cur ^ 1, cur, dc.data_ptr(), 0, stream=sp)
    e1.record(pstream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1) / rounds
    for t in trackers:
        t.close()
    return {"streams": nstreams, "sizes": {"%dx%d" % sizes[i]: int((pick == i).sum()) for i in range(3)},
            "cells_per_step": cells, "frames": steps, "cells_per_s": cells * steps / (ms.sum() / 1e3),
            "ms_per_step": float(ms.mean()), "p50_ms_per_step": float(np.percentile(ms, 50)),
            "p99_ms_per_step": float(np.percentile(ms, 99)),
            "plain": {"cells_per_s": cells / (plain_ms / 1e3), "ms_per_round": plain_ms,
                      "form": "one vtg_build + vtg_cells per frame pair, the 64 streams in turn on one stream"},
            "batched_vs_plain": (cells * steps / (ms.sum() / 1e3)) / (cells / (plain_ms / 1e3)),
            "autotune": {"chosen": tuned, "chosen_ms": tuned_ms, "default": default_tune, "default_ms": default_ms}}


def served_256(vtg, torch, ctx, pairs_1080) -> dict:
    """The served configuration at its upper end: 256 streams on Poisson schedules, two 1920x1080 at 60 fps with their
    cells on level 1 (4,080 cells), one 1280x720 at 15 fps, and 253 of 640x480 at 30 fps (2,400 cells), all with 2 %
    of frames followed by an appearance search. At nominal rates and at saturation (every stream at 200 fps), the
    served loop (continuous batching, two steps in flight) against the plain one (one frame pair at a time); at
    saturation also with LIVE priority, where frames queued behind a newer one are skipped and counted."""
    import vtg_synth as S

    small = [S.warp_pair(640, 480, S.seeded_shift(300 + k, 0), 0.5, seed=300 + k)[:2] for k in range(8)]
    p720 = S.warp_pair(1280, 720, S.seeded_shift(310, 0), 0.5, seed=310)[:2]
    pin = lambda f: torch.from_numpy(np.ascontiguousarray(f)).pin_memory()
    small_p = [(pin(a), pin(b)) for a, b in small]
    big_p = [(pin(a), pin(b)) for a, b in pairs_1080[:2]]
    p720_p = (pin(p720[0]), pin(p720[1]))
    lkcfg = vtg.config(64, 64, levels=LEVELS, cell_w=CELL_W, cell_h=CELL_H)

    def streams(rate, frames_at):
        # the cameras connect over the first half second (stream k at k / 512 s), as a server sees them come
        out, ptrs = [], []
        for k in range(2):
            out.append(dict(width=1920, height=1080, flow_level=1, fps=rate or 60.0, start_s=k / 512.0,
                            frames=frames_at(rate or 60.0)))
            ptrs += [big_p[k][0].data_ptr(), big_p[k][1].data_ptr()]
        out.append(dict(width=1280, height=720, fps=rate or 15.0, start_s=2 / 512.0, frames=frames_at(rate or 15.0)))
        ptrs += [p720_p[0].data_ptr(), p720_p[1].data_ptr()]
        for k in range(253):
            out.append(dict(width=640, height=480, fps=rate or 30.0, start_s=(3 + k) / 512.0,
                            frames=frames_at(rate or 30.0)))
            a, b = small_p[k % len(small_p)]
            ptrs += [a.data_ptr(), b.data_ptr()]
        return out, ptrs

    keys = ("cells_per_s", "p50_ms", "p99_ms", "max_ms", "mean_batch", "served", "requests", "skipped", "dropped", "ncc")
    res = {"streams": "2x1920x1080@60 (level 1, 4,080 cells), 1x1280x720@15, 253x640x480@30 (2,400 cells); "
                      "2 % of frames searched; streams start over the first 0.5 s"}
    nominal, ptrs = streams(None, lambda fps: max(2, int(round(2.0 * fps))))
    for name, plain in (("served", False), ("plain", True)):
        st = vtg.serve(ctx, nominal, ptrs, lkcfg, duration_s=2.5, max_batch=256, inflight=2, ncc_share=0.02,
                       plain=plain, seed=21)
        res.setdefault("nominal", {})[name] = {k: st[k] for k in keys}
    sat, ptrs = streams(200.0, lambda fps: 200)
    for name, plain, live in (("served", False, False), ("plain", True, False), ("served_live", False, True)):
        st = vtg.serve(ctx, sat, ptrs, lkcfg, duration_s=1.0, max_batch=256, inflight=2, ncc_share=0.02,
                       plain=plain, live=live, seed=22, allow_timeout=True)
        res.setdefault("saturation", {})[name] = {k: st[k] for k in keys}
        res["saturation"][name]["rc"] = st["rc"]
    n, s_ = res["nominal"], res["saturation"]
    res["nominal"]["served_vs_plain_cells_per_s"] = n["served"]["cells_per_s"] / max(n["plain"]["cells_per_s"], 1e-9)
    res["saturation"]["served_vs_plain_cells_per_s"] = s_["served"]["cells_per_s"] / max(s_["plain"]["cells_per_s"],
                                                                                         1e-9)
    return res


def run_ours(args) -> dict | None:
    import torch

    import vtg
    import vtg_build

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    device = f"cuda:{local}"
    vtg_build.build()
    B = args.streams
    pairs = frames_1080(B)
    dev = [(torch.from_numpy(f0).to(device), torch.from_numpy(f1).to(device)) for f0, f1 in pairs]
    torch.cuda.synchronize()
    ctx = vtg.Context(local)
    clk = Clocks(local).__enter__()

    # ---- the plain GPU form
    plain = time_plain(vtg, torch, ctx, dev, max(args.steps, 24), args.warmup, device)

    # ---- the batched form: B streams a step, autotuned, replayed from CUDA graphs
    trackers = [vtg.Tracker(ctx, vtg.config(W, H, levels=LEVELS, cell_w=CELL_W, cell_h=CELL_H)) for _ in range(B)]
    batch = vtg.Batch(ctx, B)
    batch.prepare(0, trackers, [d0.data_ptr() for d0, _ in dev], [0] * B)
    batch.prepare(1, trackers, [d1.data_ptr() for _, d1 in dev], [1] * B)
    batch.launch(0)
    batch.launch(1)
    ctx.sync()
    default_tune = batch.get_tune()
    tuned, tuned_ms, default_ms = batch.autotune(1, reps=5)
    batch.capture(0)
    batch.capture(1)
    bstream = torch.cuda.ExternalStream(batch.stream)
    for k in range(args.warmup):
        batch.replay(k & 1)
    ctx.sync()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    for k in range(args.steps):
        ev[k][0].record(bstream)
        batch.replay((args.warmup + k) & 1)
        ev[k][1].record(bstream)
    torch.cuda.synchronize()
    step_ms = np.array([a.elapsed_time(b) for a, b in ev])
    total_ms = float(step_ms.sum())
    total_ms = max_over_ranks(total_ms, device)
    value = whole_job_cells_per_s(world, B, CELLS, args.steps, total_ms)

    # ---- rooflines: the LK launch and the pyramid launches of a batched step, timed apart
    pyr_ms, lk_ms = batch.profile(1, reps=7)
    work = batch.count(1)
    flops = lk_flops(work)
    pk = peaks()
    sm_max = pk.get("sm_max_mhz", 2070.0)
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = sms * 128 * 2 * sm_max * 1e6 / 1e12
    achieved = flops / (lk_ms / 1e3) / 1e12
    roofline = {"kernel": "lk_batch_kernel", "bound": "fp32", "achieved": achieved, "peak": fp32_peak,
                "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                "peak_source": "nominal FP32 CUDA-core rate (%d SMs x 128 lanes x 2) at the measured max SM clock "
                               "(MEASURED_PEAKS.json sm_max_mhz); MEASURED_PEAKS.json holds no FP32 rate" % sms,
                "algorithmic_flop_per_launch": flops, "work_per_launch": work, "launch_ms": lk_ms,
                "traffic": LK_TRAFFIC_BYTES * B / 8,
                "traffic_source": "constant: ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of this "
                                  "step (8 streams, scaled by streams / 8), captured apart from this run",
                "traffic_note": "the algorithmic bytes are the streams' two pyramid sets read once plus the cell "
                                "records written"}
    # algorithmic bytes of a frame's pyramid: the bytes read once, the levels above 0 as 16-bit Q6, and, as level 0 is
    # materialised, 2 W H more; the build stores every level, level 0 included, as F32 (the LK kernel's loads need no
    # conversion), which is what it writes
    levels = [(1920, 1080), (960, 540), (480, 270), (240, 135)]
    pyr_bytes = B * (W * H + 2 * sum(a * b for a, b in levels[1:]) + 2 * W * H)
    pyr_stored = B * (W * H + 4 * sum(a * b for a, b in levels))
    hbm = pk.get("hbm_gbs", 6800.0)
    roof_pyr = {"kernel": "pyr_fused_batch_kernel (levels 0-3 of all streams, 1 launch a step)", "bound": "hbm",
                "achieved": pyr_bytes / (pyr_ms / 1e3) / 1e9, "peak": hbm, "unit": "GB/s",
                "frac": pyr_bytes / (pyr_ms / 1e3) / 1e9 / hbm,
                "algorithmic_bytes_per_step": pyr_bytes,
                "algorithmic_bytes_note": "per frame W H bytes read + 2 bytes a pixel of every level (16-bit Q6, "
                                          "level 0 materialised)",
                "stored_bytes_per_step": pyr_stored, "stored_frac": pyr_stored / (pyr_ms / 1e3) / 1e9 / hbm,
                "stored_bytes_note": "what the build moves: the bytes read + every level written as F32",
                "ms_per_step": pyr_ms,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in pk else "fallback 6.8 TB/s"}
    batch.close()
    for t in trackers:
        t.close()
    mix64 = time_batched_mix(vtg, torch, ctx, device)
    ncc = ncc_config3(vtg, torch, ctx)
    s256 = served_256(vtg, torch, ctx, pairs)

    # ---- end to end: the served loop through the C ABI, pinned host frames in, cell records out
    pinned = []
    for f0, f1 in pairs:
        pinned += [torch.from_numpy(f0).pin_memory(), torch.from_numpy(f1).pin_memory()]
    lkcfg = vtg.config(64, 64, levels=LEVELS, cell_w=CELL_W, cell_h=CELL_H)
    frames_per_stream = max(60, args.steps * 4)
    sat = [dict(width=W, height=H, fps=1000.0, start_s=0.0, frames=frames_per_stream) for _ in range(B)]
    served = vtg.serve(ctx, sat, [p.data_ptr() for p in pinned], lkcfg, duration_s=10.0, max_batch=B, inflight=2,
                       ncc_share=0.02, seed=11)
    served_plain = vtg.serve(ctx, sat, [p.data_ptr() for p in pinned], lkcfg, duration_s=30.0, max_batch=B,
                             inflight=1, ncc_share=0.02, plain=True, seed=11)
    e2e = {"value": served["cells_per_s"], "unit": "cells/s", "h2d_bytes_per_step": W * H,
           "d2h_bytes_per_step": CELLS * 24, "step": "one frame pair (new frame in, its 16,200 cell records out)",
           "p50_ms_per_pair": served["p50_ms"], "p99_ms_per_pair": served["p99_ms"], "mean_batch": served["mean_batch"],
           "ncc_searches": served["ncc"], "arrivals": "Poisson, %d streams x 1000 fps (saturating)" % B}
    e2e_plain = {"value": served_plain["cells_per_s"], "unit": "cells/s", "p50_ms_per_pair": served_plain["p50_ms"],
                 "p99_ms_per_pair": served_plain["p99_ms"]}
    # latency below saturation: the same streams at a camera's 30 fps (240 frame pairs/s offered)
    live = [dict(width=W, height=H, fps=30.0, start_s=0.0, frames=150) for _ in range(B)]
    lat = vtg.serve(ctx, live, [p.data_ptr() for p in pinned], lkcfg, duration_s=5.0, max_batch=B, inflight=2,
                    ncc_share=0.02, seed=13)
    lat_plain = vtg.serve(ctx, live, [p.data_ptr() for p in pinned], lkcfg, duration_s=5.0, max_batch=B,
                          inflight=1, ncc_share=0.02, plain=True, seed=13)
    e2e_latency = {"arrivals": "Poisson, %d streams x 30 fps of 1920x1080" % B,
                   "served": {k: lat[k] for k in ("cells_per_s", "p50_ms", "p99_ms", "mean_batch", "served")},
                   "plain": {k: lat_plain[k] for k in ("cells_per_s", "p50_ms", "p99_ms", "served")}}
    # nominal rates, mixed sizes: two 1080p at 60 fps (4,080 cells at level 1), one 720p at 15 fps, 13 more
    mix = [dict(width=1920, height=1080, flow_level=1, fps=60.0, start_s=0.0, frames=90),
           dict(width=1920, height=1080, flow_level=1, fps=60.0, start_s=0.0, frames=90),
           dict(width=1280, height=720, fps=15.0, start_s=0.0, frames=25)]
    sizes = [(640, 480), (1280, 720), (1920, 1080)]
    for k in range(13):
        w, h = sizes[k % 3]
        mix.append(dict(width=w, height=h, fps=30.0, start_s=0.05 * k, frames=45))
    mix_frames = []
    for k, s in enumerate(mix):
        src = pairs[k % B]
        for f in src:
            mix_frames.append(torch.from_numpy(np.ascontiguousarray(f[:s["height"], :s["width"]])).pin_memory())
    mixed = vtg.serve(ctx, mix, [p.data_ptr() for p in mix_frames], lkcfg, duration_s=3.0, max_batch=32, inflight=2,
                      ncc_share=0.02, seed=12)
    mixed_plain = vtg.serve(ctx, mix, [p.data_ptr() for p in mix_frames], lkcfg, duration_s=3.0, max_batch=32,
                            inflight=1, ncc_share=0.02, plain=True, seed=12)
    clk.__exit__(None, None, None)
    ctx.close()
    if rank != 0:
        return None
    line = {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded noise, blur 1.5, warp)",
            "config": workload("batched, graph-replayed", B),
            "p50_ms_per_step": float(np.percentile(step_ms, 50)), "p99_ms_per_step": float(np.percentile(step_ms, 99)),
            "plain": plain, "batched_vs_plain": value / plain["value"],
            "autotune": {"chosen": tuned, "chosen_ms": tuned_ms, "default_ms": default_ms,
                         "default": default_tune},
            "e2e": e2e, "e2e_plain": e2e_plain, "e2e_vs_plain": e2e["value"] / max(e2e_plain["value"], 1e-9),
            "e2e_latency": e2e_latency, "batched_mix64": mix64,
            "served_mix": {"served": {k: mixed[k] for k in ("cells_per_s", "p50_ms", "p99_ms", "mean_batch", "ncc",
                                                            "served")},
                           "plain": {k: mixed_plain[k] for k in ("cells_per_s", "p50_ms", "p99_ms", "served")},
                           "streams": "2x1080p@60 (4,080 cells), 1x720p@15, 13 more 640x480..1080p@30"},
            # a batched step: one pyramid launch for each level above 0, then one LK launch
            "served_256": s256,
            "roofline": roofline, "roofline_pyramid": roof_pyr, "ncc": ncc,
            "gpu_launches": args.steps * ((LEVELS - 1) + 1),
            "clocks": clk.summary()}
    line["cpu_baseline"] = cpu_baseline(pairs[0])
    return line


def cpu_model() -> str:
    """The host CPU as /proc/cpuinfo names it (model name on x86; implementer / part on Arm), with its core count."""
    import platform

    model = ""
    try:
        with open("/proc/cpuinfo") as f:
            info = f.read()
        for line in info.splitlines():
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
        if not model:
            impl = [l.split(":", 1)[1].strip() for l in info.splitlines() if l.startswith("CPU implementer")]
            part = [l.split(":", 1)[1].strip() for l in info.splitlines() if l.startswith("CPU part")]
            if impl and part:
                model = "Arm implementer %s part %s" % (impl[0], part[0])
    except OSError:
        pass
    return "%s, %s, %d cores" % (model or "unknown", platform.machine(), os.cpu_count() or 1)


REF_BENCH = os.path.join(ORACLE, "_ref", "vtref_bench")


def reference_bench(frames, steps: int, warmup: int, threads: int, lk: str = "ref", pyr: str = "ref",
                    every: int = 1, interleave: int = 0) -> dict | None:
    """Runs oracle/_ref/vtref_bench, the reference's own pyramid and LK kernels (its C sources, built on this host by
    oracle/Makefile) on the workload's frame pair and its 16,200 cell centres; None where it is not built."""
    import tempfile

    sys.path.insert(0, ORACLE)
    import oracle as O

    if not os.path.exists(REF_BENCH):
        subprocess.run(["make", "-s", "-C", ORACLE, "refbin"], capture_output=True)
    if not os.path.exists(REF_BENCH):
        return None
    f0, f1 = frames
    xs, ys = O.cell_centres(W, H, CELL_W, CELL_H)
    with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as f:
        f.write(np.array([W, H, LEVELS, len(xs)], np.int32).tobytes())
        f.write(np.ascontiguousarray(f0, np.uint8).tobytes())
        f.write(np.ascontiguousarray(f1, np.uint8).tobytes())
        f.write(np.asarray(xs, np.float32).tobytes())
        f.write(np.asarray(ys, np.float32).tobytes())
        path = f.name
    try:
        cmd = [REF_BENCH, path, "--lk", lk, "--pyr", pyr, "--threads", str(threads), "--steps", str(steps),
               "--warmup", str(warmup), "--every", str(every)]
        if interleave:
            cmd += ["--interleave", str(interleave)]
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
        if r.returncode != 0:
            return None
        return json.loads(r.stdout.strip().splitlines()[-1])
    finally:
        os.unlink(path)


def cpu_baseline(frames, seconds: float = 10.0) -> dict:
    """The reference's own CPU code on all host cores: its plain-C pyramid (img_u8_to_q6_ref, img_reduce_ref) and LK
    with the forward-backward check (lk_track_ref, lk_flowback_ref) over the workload's 16,200 cells, frame pairs
    repeated for about `seconds`. Where that build is missing, the oracle's FP64 restatement instead (kind "port")."""
    threads = os.cpu_count() or 1
    probe = reference_bench(frames, 1, 1, threads)
    if probe is not None:
        steps = max(2, int(seconds / max(probe["median_s"], 1e-3)))
        r = reference_bench(frames, steps, 1, threads)
        if r is not None:
            return {"value": r["cells_per_s"], "unit": "cells/s", "cores": threads, "kind": "reference",
                    "sample": "%d whole frame pairs (pyramid + 16,200 cells with flowback) in %.1f s: the reference's "
                              "img_*_ref + lk_track_ref / lk_flowback_ref built from its sources, on %s"
                              % (steps, r["total_s"], cpu_model())}
    sys.path.insert(0, ORACLE)
    import oracle as O

    f0, f1 = frames
    xs, ys = O.cell_centres(W, H, CELL_W, CELL_H)
    xs, ys = xs[::4], ys[::4]
    cfg = O.lk_cfg()
    P0 = O.pyramid(f0, LEVELS)
    done, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        P1 = O.pyramid(f1, LEVELS)
        O.lk_points(P0, P1, LEVELS - 1, cfg, xs, ys, max_fb=0.5, mode=O.F64, threads=threads)
        done += len(xs)
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": "cells/s", "cores": threads, "kind": "port",
            "sample": "the reference's own build is missing here: the new frame's pyramid + every 4th of the 16,200 "
                      "cells per repetition, FP64 oracle form, %d repetitions in %.1f s on %s"
                      % (done // len(xs), dt, cpu_model())}


def run_reference(args) -> dict | None:
    """The reference arm: the reference's own CPU implementation of the path (its C kernels, built from its sources on
    this host) on all host cores, K timed steps after W warm-up steps, a step being one frame pair of this bench's
    workload (the new frame's pyramid and LK with flowback at all 16,200 cells). Beside it, the reference's vector
    kernels (their 16-lane host model) against the plain C ones, median of 7 interleaved rounds on every 8th cell."""
    if int(os.environ.get("RANK", "0")) != 0:
        return None
    import vtg_synth as S

    threads = os.cpu_count() or 1
    frames = S.warp_pair(W, H, S.seeded_shift(2, 0), 0.5, seed=2)[:2]
    r = reference_bench(frames, args.steps, args.warmup, threads)
    if r is None:
        return run_reference_port(args, frames)
    inter = reference_bench(frames, 1, 0, threads, every=8, interleave=7)
    value = r["cells_per_s"]
    cb = {"value": value, "unit": "cells/s", "cores": threads, "kind": "reference",
          "sample": "per step one whole frame pair: the reference's img_u8_to_q6_ref + img_reduce_ref pyramid and "
                    "lk_track_ref + lk_flowback_ref at all 16,200 cells, its C sources built on this host, "
                    "threads over an atomic cell counter, on %s" % cpu_model()}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * r["total_s"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 patch sums, long double driver",
            "data": "synthetic (seeded noise, blur 1.5, warp)", "config": workload("batched, graph-replayed",
                                                                                args.streams),
            "cpu_baseline": cb, "median_ms_per_step": 1e3 * r["median_s"],
            "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if inter is not None:
        line["vector_kernels"] = {"what": "the reference's _vx kernels (its 16-lane host model) against its plain C "
                                          "ones, median of 7 interleaved rounds on every 8th cell",
                                  "ref_cells_per_s": inter["ref_cells_per_s"], "vx_cells_per_s": inter["vx_cells_per_s"]}
    return line


def run_reference_port(args, frames) -> dict:
    """The reference arm where the reference's own build is missing: the oracle's FP64 restatement of its path."""
    sys.path.insert(0, ORACLE)
    import oracle as O

    threads = os.cpu_count() or 1
    f0, f1 = frames
    xs, ys = O.cell_centres(W, H, CELL_W, CELL_H)
    xs, ys = xs[::8], ys[::8]
    cfg = O.lk_cfg()
    P0 = O.pyramid(f0, LEVELS)

    def step():
        P1 = O.pyramid(f1, LEVELS)
        O.lk_points(P0, P1, LEVELS - 1, cfg, xs, ys, max_fb=0.5, mode=O.F64, threads=threads)

    for _ in range(args.warmup):
        step()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = len(xs) * args.steps / total
    cb = {"value": value, "unit": "cells/s", "cores": threads, "kind": "port",
          "sample": "the reference's own build is missing here: per step one stream's new frame's pyramid and every "
                    "8th cell (2,025 of 16,200), FP64 oracle form, all host threads, %s" % cpu_model()}
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded noise, blur 1.5, warp)", "config": workload("batched, graph-replayed",
                                                                                args.streams),
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def ncc_config3(vtg, torch, ctx, templates: int = 10, reps: int = 5) -> dict:
    """The whole-picture appearance search at the NCC configuration: a seeded 1920 x 1080 8-bit frame, templates of 32,
    64 and 96 cut at seeded corners and perturbed (gain 0.8-1.2, offset +-20, noise sigma 3), one in ten near-blank
    (standard deviation below 2), step 1, per map precision (F32 on CUDA cores, BF16 and FP16 on the tensor cores).
    Per size and precision: the CUDA-event time of the map kernel alone and of the whole search (window sums, map,
    eight candidates, half-pixel re-score; median over the templates of the median of `reps` runs), the map's useful
    FLOP rate (2 T^2 per corner) and its fraction of the measured BF16 burst rate, the found corner against the true one
    and the F32 map's, the score against the FP64 oracle at the found half-pixel corner, and the near-blank templates'
    best scores (a match would be 0.5 or more)."""
    sys.path.insert(0, ORACLE)
    import oracle as O
    import vtg_synth as S

    frame = S.noise_frame(W, H, seed=3)
    fplane = frame.astype(np.float32)
    d = torch.from_numpy(frame).cuda()
    torch.cuda.synchronize()
    s = vtg.Search(ctx, W, H)
    pk = peaks()
    peak = pk.get("bf16_tflops", 1900.0)
    names = ((vtg.NCC_F32, "f32"), (vtg.NCC_BF16, "bf16"), (vtg.NCC_FP16, "fp16"))
    out = {"frame": "%dx%d u8, seeded blurred noise" % (W, H), "templates_per_size": templates, "step": 1,
           "peak_bf16_tflops": peak,
           "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst; of measured)" if "bf16_tflops" in pk else
           "fallback 1.9 PFLOP/s", "sizes": {}}
    for size in (32, 64, 96):
        tpl, xs, ys, blank = S.ncc_templates(frame, size, templates, seed=size, blank_share=0.1)
        corners = (W - size - 2) * (H - size - 2)
        rows = {name: {"map_ms": [], "search_ms": [], "found_true": 0, "agree_f32": 0, "err_fp64": 0.0,
                       "blank_best": []} for _, name in names}
        for k in range(templates):
            app = (tpl[k].astype(np.float32) - np.float32(tpl[k].mean(dtype=np.float64))).astype(np.float32)
            norm = float(np.sum(app.astype(np.float64) ** 2))
            s.template(app, norm)
            f32 = None
            for prec, name in names:
                f = s.run(d.data_ptr(), W, H, W, vtg.PLANE_U8, 1, W, 1, H, 1, prec)
                f32 = f if prec == vtg.NCC_F32 else f32
                mms, tms = s.profile(d.data_ptr(), W, H, W, vtg.PLANE_U8, 1, W, 1, H, 1, prec,
                                     reps=3 if prec == vtg.NCC_F32 else reps)
                r = rows[name]
                r["map_ms"].append(mms)
                r["search_ms"].append(tms)
                if blank[k]:
                    r["blank_best"].append(f["ncc"])
                    continue
                r["found_true"] += int((f["hx"], f["hy"]) == (2 * int(xs[k]), 2 * int(ys[k])))
                r["agree_f32"] += int((f["hx"], f["hy"]) == (f32["hx"], f32["hy"]))
                o = O.ncc_half(fplane, app, norm, f["hx"], f["hy"], O.F64)
                r["err_fp64"] = max(r["err_fp64"], abs(f["ncc"] - o))
        res = {}
        nb = int(blank.sum())
        for _, name in names:
            r = rows[name]
            map_ms = float(np.median(r["map_ms"]))
            tflops = 2.0 * size * size * corners / (map_ms / 1e3) / 1e12
            res[name] = {"map_ms": map_ms, "search_ms": float(np.median(r["search_ms"])),
                         "map_tflops_useful": tflops, "frac_of_bf16_burst": tflops / peak,
                         "found_true": "%d/%d" % (r["found_true"], templates - nb),
                         "agree_with_f32": "%d/%d" % (r["agree_f32"], templates - nb),
                         "max_score_err_vs_fp64": r["err_fp64"],
                         "near_blank": {"templates": nb, "best_scores": r["blank_best"],
                                        "matched": int(sum(v >= 0.5 for v in r["blank_best"]))}}
        out["sizes"][str(size)] = res
    s.close()
    return out


def run_ncc(args) -> dict:
    """`--ncc`: the appearance search at the NCC configuration alone (see ncc_config3)."""
    import torch

    import vtg
    import vtg_build

    vtg_build.build()
    ctx = vtg.Context(0)
    out = {"metric": "appearance search ms per template (whole 1920x1080 picture, step 1)", "unit": "ms",
           "higher_is_better": False, **ncc_config3(vtg, torch, ctx)}
    ctx.close()
    return out


def run_detect(args) -> dict:
    """Corner detection (seed_at's detect_begin .. detect_finish) on level 0 of a 1080p frame: a 384 x 307 box (the size
    the reference times on the card: 3.78 ms on its thread team) and the whole frame. CUDA-event time of the whole
    detection, the response kernel's share, and the FP64-free selection; the oracle's CPU time beside it; the corners
    against the oracle's."""
    import torch

    import vtg
    import vtg_build

    sys.path.insert(0, ORACLE)
    import oracle as O

    vtg_build.build()
    f0, _, _, _ = __import__("vtg_synth").warp_pair(W, H, __import__("vtg_synth").seeded_shift(2, 0), 0.5, seed=2)
    plane = O.pyramid(f0, 1)[0]
    d = torch.from_numpy(plane).cuda()
    torch.cuda.synchronize()
    ctx = vtg.Context(0)
    det = vtg.Detector(ctx, W, H)
    stream = torch.cuda.ExternalStream(vtg.lib().vtg_detector_stream(det.h))
    out = {"metric": "corner detection ms per region (Harris response, cells, selection) on a 1920x1080 Q6 plane",
           "unit": "ms", "higher_is_better": False, "results": []}
    pk = peaks()
    for name, (rx, ry, rw, rh, mx, md, q) in (("box 384x307", (700.5, 400.25, 384, 307, 128, 8.0, 0.05)),
                                              ("whole frame", (0, 0, W, H, 512, 10.0, 0.01))):
        args_ = (d.data_ptr(), W, H, W, rx, ry, rw, rh, 12, mx, md, q)
        xs, ys = det.detect(*args_)
        reps = 20
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        xd = torch.empty(512, device="cuda")
        yd = torch.empty(512, device="cuda")
        cd = torch.empty(1, dtype=torch.int32, device="cuda")
        for a, b in ev:
            a.record(stream)
            vtg.check(vtg.lib().vtg_detect(det.h, d.data_ptr(), W, H, W, rx, ry, rw, rh, 12, mx, md, q, xd.data_ptr(),
                                           yd.data_ptr(), cd.data_ptr(), vtg.DEVICE, None), "vtg_detect")
            b.record(stream)
        torch.cuda.synchronize()
        ms = float(np.median([a.elapsed_time(b) for a, b in ev]))
        g = O.detect_geometry(W, H, rx, ry, rw, rh, 12)
        t0 = time.perf_counter()
        oxs, oys = O.detect(plane, rx, ry, rw, rh, 12, mx, md, q)
        cpu_ms = 1e3 * (time.perf_counter() - t0)
        # the response pass reads the plane tile once and writes the response: its algorithmic bytes
        resp_bytes = 4 * (g.rows + 4) * (g.cols + 4) + 4 * g.rows * g.cols
        out["results"].append({"region": name, "rows": g.rows, "cols": g.cols, "corners": int(len(xs)), "ms": ms,
                               "same_as_oracle": bool(np.array_equal(xs, oxs) and np.array_equal(ys, oys)),
                               "cpu_oracle_ms_1_thread": cpu_ms, "response_algorithmic_bytes": resp_bytes})
    det.close()
    ctx.close()
    out["hbm_gbs"] = pk.get("hbm_gbs")
    return out


def run_points(args) -> dict:
    """The feature list path (OP_LK, track.c:275-292): LK with the forward-backward check for a list of points between
    a tracker's two pyramid sets (vtg_points), at the tracker's sizes: 128 and 512 features at 640 x 480 (3 levels,
    the reference's card: 245 us a frame for its feature list, docs/measurements.md:156), 512 and 2,048 at 1920 x 1080
    (4 levels).
    CUDA-event time of one call with its arrays in device memory, with one and with two warps a point (the warps-a-point
    choice) and with the default (one); flow (the default's) against the FP64 oracle on the points both call good; the
    oracle's time (all host cores) beside it."""
    import torch

    import vtg
    import vtg_build

    sys.path.insert(0, ORACLE)
    import oracle as O

    S = __import__("vtg_synth")
    vtg_build.build()
    ctx = vtg.Context(0)
    L = vtg.lib()
    cores = os.cpu_count() or 1
    out = {"metric": "feature-list LK ms a call (21x21, <=10 iterations, flowback 0.5)", "unit": "ms",
           "higher_is_better": False, "results": []}
    for w, h, levels, n in ((640, 480, 3, 128), (640, 480, 3, 512), (1920, 1080, 4, 512), (1920, 1080, 4, 2048)):
        f0, f1, _, _ = S.warp_pair(w, h, (3.2, -1.7), 0.5, seed=5)
        t = vtg.Tracker(ctx, vtg.config(w, h, levels=levels, fb_max=0.5))
        t.build(0, f0)
        t.build(1, f1)
        t.sync()
        u = S.uniform(5, 77, 2 * n)
        xs = (20.0 + u[:n] * (w - 40)).astype(np.float32)
        ys = (20.0 + u[n:] * (h - 40)).astype(np.float32)
        dx = torch.from_numpy(xs).cuda()
        dy = torch.from_numpy(ys).cuda()
        dout = torch.zeros(n * 32, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        stream = torch.cuda.ExternalStream(t.stream)

        def timed(warps):
            t.set_point_warps(warps)
            for _ in range(3):
                vtg.check(L.vtg_points(t.h, 0, 1, -1, n, dx.data_ptr(), dy.data_ptr(), None, None, dout.data_ptr(),
                                       vtg.DEVICE, None), "vtg_points")
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(20)]
            for e0, e1 in ev:
                e0.record(stream)
                L.vtg_points(t.h, 0, 1, -1, n, dx.data_ptr(), dy.data_ptr(), None, None, dout.data_ptr(), vtg.DEVICE,
                             None)
                e1.record(stream)
            torch.cuda.synchronize()
            return float(np.median([e0.elapsed_time(e1) for e0, e1 in ev]))

        ms_by_warps = {w_: timed(w_) for w_ in (1, 2)}
        ms = timed(0)  # the default: one warp a point
        got = dout.cpu().numpy().view(vtg.LK_OUT_DTYPE)
        I, J = O.pyramid(f0, levels), O.pyramid(f1, levels)
        t0 = time.perf_counter()
        ref = O.lk_points(I, J, levels - 1, O.lk_cfg(21, 21, 10, 0.01, 0.1, 25.0), xs, ys, max_fb=0.5, mode=O.F64,
                          threads=cores)
        cpu_ms = 1e3 * (time.perf_counter() - t0)
        both = (got["status"] == 0) & (ref["status"] == 0)
        err = float(np.max(np.maximum(np.abs(got["x"] - ref["x"]), np.abs(got["y"] - ref["y"]))[both])) if both.any() else None
        out["results"].append({"frame": "%dx%d" % (w, h), "levels": levels, "points": n, "ms": ms,
                               "ms_one_warp_a_point": ms_by_warps[1], "ms_two_warps_a_point": ms_by_warps[2],
                               "status_agreement": float(np.mean(got["status"] == ref["status"])),
                               "max_err_px": err, "cpu_oracle_ms": cpu_ms, "cpu_cores": cores,
                               "reference_card_us": 245 if w == 640 else None})
        t.close()
    ctx.close()
    return out


def run_build(args) -> dict:
    """tk_build with its optional input steps (track.c:584-629): the pyramid of one 8-bit frame from device memory
    (vtg_build) with neither, the contrast stretch, the 5 x 5 binomial, or both, at 640 x 480 (3 levels), 1280 x 720
    and 1920 x 1080 (4 levels). CUDA-event time of one call; every level checked against the oracle; the oracle's own
    time (one host thread) beside it. Algorithmic bytes: the frame read once and every level written once (F32), plus
    level 0 read once more by the reduce when an input step made it."""
    import torch

    import vtg
    import vtg_build

    sys.path.insert(0, ORACLE)
    import oracle as O

    S = __import__("vtg_synth")
    vtg_build.build()
    ctx = vtg.Context(0)
    L = vtg.lib()
    out = {"metric": "tk_build ms a frame (pyramid with the optional input steps)", "unit": "ms",
           "higher_is_better": False, "results": []}
    for w, h, levels in ((640, 480, 3), (1280, 720, 4), (1920, 1080, 4)):
        f = S.build_frame("low", w, h, 11)
        d = torch.from_numpy(f).cuda()
        torch.cuda.synchronize()
        t = vtg.Tracker(ctx, vtg.config(w, h, levels=levels))
        stream = torch.cuda.ExternalStream(t.stream)
        for opts, name in ((0, "plain"), (1, "contrast"), (2, "pre_gauss"), (3, "contrast+pre_gauss")):
            t.set_build(opts)
            for _ in range(3):
                vtg.check(L.vtg_build(t.h, 0, d.data_ptr(), w, vtg.DEVICE, None), "vtg_build")
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(20)]
            for e0, e1 in ev:
                e0.record(stream)
                L.vtg_build(t.h, 0, d.data_ptr(), w, vtg.DEVICE, None)
                e1.record(stream)
            torch.cuda.synchronize()
            ms = float(np.median([e0.elapsed_time(e1) for e0, e1 in ev]))
            t0 = time.perf_counter()
            want = O.pyramid(f, levels, opts)
            cpu_ms = 1e3 * (time.perf_counter() - t0)
            exact = all(np.array_equal(t.level(0, k), want[k]) for k in range(levels))
            dims = O.level_dims(w, h, levels)
            nbytes = w * h + 4 * sum(a * b for a, b in dims) + (4 * w * h if opts else 0)
            out["results"].append({"frame": "%dx%d" % (w, h), "levels": levels, "steps": name, "ms": ms,
                                   "gbs": nbytes / (ms * 1e-3) / 1e9, "bit_exact": exact, "cpu_oracle_ms": cpu_ms,
                                   "cpu_cores": 1})
        t.close()
    ctx.close()
    return out


def run_still(args) -> dict:
    """The still picture (still_vectors, still_decide, still_update, still_finish) a frame, on a 12-frame sequence at
    level 1 of a 1080p camera (960 x 540, 4,080 cells) and at native 1080p (16,200 cells): CUDA-event time of a whole
    frame and of the decision and update alone (the frame's cells fed from device memory), the oracle's CPU time a
    frame beside it. The reference's card times these at 1,448 + 1,648 us (level 1) and 4,515 + 5,825 us (native):
    vectors + "mean" (docs/measurements.md:446-448)."""
    import torch

    import vtg
    import vtg_build

    sys.path.insert(0, ORACLE)
    import oracle as O

    S = __import__("vtg_synth")
    vtg_build.build()
    ctx = vtg.Context(0)
    out = {"metric": "still picture ms a frame (per-cell LK from the mean, decision, running mean)", "unit": "ms",
           "higher_is_better": False, "results": []}
    cores = os.cpu_count() or 1
    for name, (w, h), ref_us in (("level 1 of 1080p", (960, 540), (1448, 1648)),
                                 ("native 1080p", (1920, 1080), (4515, 5825))):
        seq = S.still_sequence(w, h, 12, seed=4)
        planes = [torch.from_numpy(O.pyramid(f, 1)[0]).cuda() for f in seq]
        torch.cuda.synchronize()
        st = vtg.Still(ctx, w, h, 8, 1.0, 4.0)
        stream = torch.cuda.ExternalStream(st.stream())
        for k in range(3):
            st.frame(planes[k].data_ptr(), w)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(9)]
        for k, (a, b) in enumerate(ev):
            a.record(stream)
            st.frame(planes[3 + k].data_ptr(), w)
            b.record(stream)
        torch.cuda.synchronize()
        frame_ms = float(np.median([a.elapsed_time(b) for a, b in ev]))
        cells, m, _ = st.read()
        dcells = torch.from_numpy(cells.view(np.uint8).copy()).cuda()
        torch.cuda.synchronize()
        L = vtg.lib()
        for a, b in ev:
            a.record(stream)
            vtg.check(L.vtg_still_frame(st.h, planes[11].data_ptr(), w, dcells.data_ptr(), vtg.DEVICE, None),
                      "vtg_still_frame")
            b.record(stream)
        torch.cuda.synchronize()
        mean_ms = float(np.median([a.elapsed_time(b) for a, b in ev]))
        st.close()
        # the oracle: two frames after the first, all host cores (FP64 vectors)
        ref = O.Still(w, h, 8, 1.0, 4.0)
        qs = [O.pyramid(f, 1)[0] for f in seq[:3]]
        ref.frame(qs[0])
        t0 = time.perf_counter()
        for q in qs[1:]:
            ref.frame(q, mode=O.F64, threads=cores)
        cpu_ms = 1e3 * (time.perf_counter() - t0) / 2
        ref.close()
        out["results"].append({"plane": name, "w": w, "h": h, "cells": int(len(cells)), "frame_ms": frame_ms,
                               "decide_update_ms": mean_ms, "vectors_ms": frame_ms - mean_ms,
                               "moving": int(m["moving"]), "tracked": int(m["tracked"]),
                               "cpu_oracle_ms": cpu_ms, "cpu_cores": cores,
                               "reference_card_ms": {"vectors": ref_us[0] / 1e3, "mean": ref_us[1] / 1e3}})
    ctx.close()
    return out


def run_framegen(args) -> dict:
    """Frame generation (framegen.c as tk_generate_make runs it): one generated frame between two frames of a warped
    pair, CUDA-event time of the whole call (the field's pyramid, the scene test, search, filter and upscale at every
    level, the middle vectors, the blended frame and its bytes), at 640 x 480, 1280 x 720 and 1920 x 1080. The fields
    and frame are checked against the oracle, whose time (one CPU thread) is beside it. The reference's card: 5.98 ms a
    1080p frame, 2.79 ms of it the search (docs/measurements.md:534-536); 1.68 to 1.93 ms at 640 x 480 (:532)."""
    import torch

    import vtg
    import vtg_build

    sys.path.insert(0, ORACLE)
    import oracle as O

    S = __import__("vtg_synth")
    vtg_build.build()
    ctx = vtg.Context(0)
    out = {"metric": "generated frame ms (motion field, middle vectors, blend)", "unit": "ms",
           "higher_is_better": False, "results": []}
    card = {(640, 480): 1.93, (1920, 1080): 5.977}
    for w, h in ((640, 480), (1280, 720), (1920, 1080)):
        f0, f1, _, _ = S.warp_pair(w, h, (-17.0, 12.0), 3.0, seed=8)
        a = torch.from_numpy(O.pyramid(f0, 1)[0]).cuda()
        b = torch.from_numpy(O.pyramid(f1, 1)[0]).cuda()
        dpic = torch.zeros((h, w), dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        fg = vtg.Framegen(ctx, w, h)
        stream = torch.cuda.ExternalStream(fg.stream())
        L = vtg.lib()
        for _ in range(3):
            vtg.check(L.vtg_framegen_run(fg.h, a.data_ptr(), w, b.data_ptr(), w, None, 0, dpic.data_ptr(), vtg.DEVICE,
                                         None), "vtg_framegen_run")
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(20)]
        for e0, e1 in ev:
            e0.record(stream)
            L.vtg_framegen_run(fg.h, a.data_ptr(), w, b.data_ptr(), w, None, 0, dpic.data_ptr(), vtg.DEVICE, None)
            e1.record(stream)
        torch.cuda.synchronize()
        ms = float(np.median([e0.elapsed_time(e1) for e0, e1 in ev]))
        r = fg.fields()
        pic = dpic.cpu().numpy()
        fg.close()
        t0 = time.perf_counter()
        o = O.framegen(O.pyramid(f0, 1)[0], O.pyramid(f1, 1)[0])
        cpu_ms = 1e3 * (time.perf_counter() - t0)
        same = np.array_equal(pic, o["pic"]) and all(x.tobytes() == y.tobytes() for x, y in zip(r["fil"], o["fil"]))
        out["results"].append({"frame": "%dx%d" % (w, h), "levels": len(r["fil"]), "ms": ms,
                               "same_as_oracle": bool(same), "cpu_oracle_ms_1_thread": cpu_ms,
                               "reference_card_ms": card.get((w, h))})
    ctx.close()
    return out


def run_profile(args) -> None:
    """Launches for an ncu capture, nothing timed: `batch` primes B 1080p streams (2 batched steps) and runs 2 more
    (capture lk_batch_kernel with -s 2); `ncc` runs one 1080p whole-picture search per precision (a --ncc-size
    template)."""
    import torch

    import vtg
    import vtg_build
    import vtg_synth as S

    vtg_build.build()
    ctx = vtg.Context(0)
    if args.profile == "batch":
        B = args.streams
        pairs = frames_1080(B)
        dev = [(torch.from_numpy(f0).cuda(), torch.from_numpy(f1).cuda()) for f0, f1 in pairs]
        torch.cuda.synchronize()
        trackers = [vtg.Tracker(ctx, vtg.config(W, H, levels=LEVELS, cell_w=CELL_W, cell_h=CELL_H)) for _ in range(B)]
        batch = vtg.Batch(ctx, B)
        batch.prepare(0, trackers, [d0.data_ptr() for d0, _ in dev], [0] * B)
        batch.prepare(1, trackers, [d1.data_ptr() for _, d1 in dev], [1] * B)
        for k in range(4):
            batch.launch(k & 1)
        ctx.sync()
        print("profile batch: %d streams, %d cells a step" % (B, batch.cells(0)))
    elif args.profile == "still":
        sys.path.insert(0, ORACLE)
        import oracle as O

        seq = S.still_sequence(W, H, 4, seed=4)
        planes = [torch.from_numpy(O.pyramid(f, 1)[0]).cuda() for f in seq]
        torch.cuda.synchronize()
        st = vtg.Still(ctx, W, H, 8, 1.0, 4.0)
        for p_ in planes:
            st.frame(p_.data_ptr(), W)
        _, m, _ = st.read()
        print("profile still: %d frames, %d moving" % (int(m["frames"]), int(m["moving"])))
        st.close()
    elif args.profile == "framegen":
        sys.path.insert(0, ORACLE)
        import oracle as O

        f0, f1, _, _ = S.warp_pair(W, H, (-17.0, 12.0), 3.0, seed=8)
        a = torch.from_numpy(O.pyramid(f0, 1)[0]).cuda()
        b = torch.from_numpy(O.pyramid(f1, 1)[0]).cuda()
        torch.cuda.synchronize()
        fg = vtg.Framegen(ctx, W, H)
        for _ in range(2):
            fg.run(a.data_ptr(), W, b.data_ptr(), W)
        print("profile framegen: %d levels" % fg.levels)
        fg.close()
    elif args.profile == "detect":
        sys.path.insert(0, ORACLE)
        import oracle as O

        f0, _, _, _ = S.warp_pair(W, H, S.seeded_shift(2, 0), 0.5, seed=2)
        d = torch.from_numpy(O.pyramid(f0, 1)[0]).cuda()
        torch.cuda.synchronize()
        det = vtg.Detector(ctx, W, H)
        for reg in ((700.5, 400.25, 384, 307, 128, 8.0, 0.05), (0, 0, W, H, 512, 10.0, 0.01)):
            xs, ys = det.detect(d.data_ptr(), W, H, W, *reg[:4], 12, *reg[4:])
            print("profile detect: %d corners" % len(xs))
        det.close()
    else:
        frame = S.noise_frame(W, H, seed=3)
        tpl, xs, ys, _ = S.ncc_templates(frame, args.ncc_size, 1, seed=1, blank_share=0.0)
        app = (tpl[0].astype(np.float32) - np.float32(tpl[0].mean(dtype=np.float64))).astype(np.float32)
        norm = float(np.sum(app.astype(np.float64) ** 2))
        d = torch.from_numpy(frame).cuda()
        torch.cuda.synchronize()
        s = vtg.Search(ctx, W, H)
        s.template(app, norm)
        for prec in (vtg.NCC_BF16, vtg.NCC_FP16, vtg.NCC_F32):
            f = s.run(d.data_ptr(), W, H, W, vtg.PLANE_U8, 1, W, 1, H, 1, prec)
            print("profile ncc precision %d: found (%d, %d) ncc %.4f" % (prec, f["hx"], f["hy"], f["ncc"]))
        s.close()
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--streams", type=int, default=8, help="1080p streams a batched step")
    ap.add_argument("--ncc", action="store_true",
                    help="the whole-picture appearance search on a 1080p frame (32, 64, 96 templates), per precision")
    ap.add_argument("--detect", action="store_true", help="corner detection on a 1080p plane: a 384 x 307 box, the frame")
    ap.add_argument("--framegen", action="store_true",
                    help="frame generation at 640 x 480, 1280 x 720 and 1920 x 1080 (motion field, middle vectors, blend)")
    ap.add_argument("--points", action="store_true",
                    help="the feature-list LK path: 128 and 512 points at 640 x 480, 512 at 1920 x 1080")
    ap.add_argument("--build", action="store_true",
                    help="tk_build's pyramid with and without its optional input steps at 640 x 480, 720p and 1080p")
    ap.add_argument("--still", action="store_true",
                    help="the still picture a frame at 960 x 540 and 1920 x 1080 (vectors, decision, running mean)")
    ap.add_argument("--profile", default=None, choices=["batch", "ncc", "detect", "still", "framegen"],
                    help="a short run for an ncu capture: the batched step (prime, then 2 steps) or one NCC search")
    ap.add_argument("--ncc-size", type=int, default=32, help="--profile ncc: the template's side (32, 64 or 96)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.profile:
        run_profile(args)
        return
    if args.ncc:
        print(json.dumps(run_ncc(args)))
        return
    if args.detect:
        print(json.dumps(run_detect(args)))
        return
    if args.still:
        print(json.dumps(run_still(args)))
        return
    if args.points:
        print(json.dumps(run_points(args)))
        return
    if args.build:
        print(json.dumps(run_build(args)))
        return
    if args.framegen:
        print(json.dumps(run_framegen(args)))
        return
    line = run_reference(args) if args.impl == "reference" else run_ours(args)
    if line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
