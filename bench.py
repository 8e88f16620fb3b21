"""bench.py -- LK cells/s on one GB300 for the 1920 x 1080 configuration (4 levels, 16,200 cells of 16 x 8, 21 x 21
patch, <= 10 iterations, eps 0.01, forward-backward check 0.5), seeded synthetic frames.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--form plain]

A step is one frame pair of one stream: the pyramid of the new frame and the per-cell flow from the previous frame's
pyramid to it. `value` times K steps with the frames already in HBM (CUDA events on the tracker's stream, L2 flushed
before every step by writing a 256 MiB buffer, outside the timed spans). `e2e` times the same steps through the public
C ABI with host buffers: the pinned frame's upload and the cell records' download inside the timed region.
`--impl reference` times the CPU restatement of the reference's path (oracle/, FP64 form) on all host cores over the
same workload.
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
W, H, LEVELS, CELL_W, CELL_H = 1920, 1080, 4, 16, 8
PATCH = 21


def workload(form: str) -> dict:
    return {"workload": "per-cell LK flow, 1920x1080 frame pairs, 4 levels, 16,200 cells (16x8), 21x21 patch, "
                        "<=10 iters, eps 0.01, fb 0.5; form=" + form,
            "width": W, "height": H, "levels": LEVELS, "cells_per_pair": 16200, "patch": PATCH,
            "l2": "flushed before every timed step (256 MiB write)"}


class Clocks:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
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
        sm = [float(r[0]) for r in self.rows if len(r) >= 6 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 6 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 6 for i in range(4) if r[2 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def lk_flops(lk: np.ndarray, levels: int, w: int = PATCH, h: int = PATCH) -> float:
    """Algorithmic FLOPs of the cells just computed, counting the reference's patch operations (src/kern/lk_ref.c) with
    FMA = 2: build 9 (W+2)(H+2) + 20 W H per level built, iterate 14 W H per iteration, residual 12 W H; the
    forward-backward track costs the same again for the cells that ran it (its iteration count taken equal to the
    forward track's)."""
    build = 9 * (w + 2) * (h + 2) + 20 * w * h
    fwd = levels * build + 14 * w * h * lk["iters"].astype(np.float64) + 12 * w * h
    back = np.where((lk["status"] == 0) | (lk["status"] == 8), fwd, 0.0)
    return float(np.sum(fwd + back))


def peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def run_ours(args) -> dict:
    import torch

    import vtg
    import vtg_build
    import vtg_synth as S

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    vtg_build.build()
    f0, f1, _, _ = S.warp_pair(W, H, S.seeded_shift(2, 0), 0.5, seed=2)
    frames = [f0, f1]
    ctx = vtg.Context(local)
    t = vtg.Tracker(ctx, vtg.config(W, H, levels=LEVELS, cell_w=CELL_W, cell_h=CELL_H))
    n = t.cols * t.rows
    stream = torch.cuda.ExternalStream(t.stream)
    dframes = [torch.from_numpy(f).to(f"cuda:{local}") for f in frames]
    dcells = torch.empty(n * 24, dtype=torch.uint8, device=f"cuda:{local}")
    dlk = torch.empty(n * 32, dtype=torch.uint8, device=f"cuda:{local}")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    torch.cuda.synchronize()

    def step(k: int):
        cur = k & 1
        t.build(cur, dframes[cur].data_ptr(), W, where=vtg.DEVICE, stream=None)
        t.cells_device(cur ^ 1, cur, dcells.data_ptr(), dlk.data_ptr())

    t.build(0, dframes[0].data_ptr(), W, where=vtg.DEVICE)
    for k in range(1, args.warmup + 1):
        step(k)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    lk_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        wall0 = time.perf_counter()
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 255)
                starts[k].record(stream)
            cur = (args.warmup + 1 + k) & 1
            t.build(cur, dframes[cur].data_ptr(), W, where=vtg.DEVICE)
            with torch.cuda.stream(stream):
                lk_ev[k][0].record(stream)
            t.cells_device(cur ^ 1, cur, dcells.data_ptr(), dlk.data_ptr())
            with torch.cuda.stream(stream):
                lk_ev[k][1].record(stream)
                ends[k].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    step_ms = np.array([s.elapsed_time(e) for s, e in zip(starts, ends)])
    lk_ms = np.array([a.elapsed_time(b) for a, b in lk_ev])
    total_ms = float(step_ms.sum())
    if world > 1:
        tt = torch.tensor([total_ms], device=f"cuda:{local}")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(tt.item())
    value = world * n * args.steps / (total_ms / 1e3)

    # end to end through the C ABI: pinned host frame in, cell records out, every step
    if args.skip_e2e:
        t.close()
        ctx.close()
        return {"metric": METRIC, "value": value, "unit": "cells/s", "ms_per_step": total_ms / args.steps,
                "lk_ms": float(lk_ms.mean()), "note": "profiling run: e2e and baselines skipped"} if rank == 0 else None
    pinned = [torch.from_numpy(f).pin_memory() for f in frames]
    host_cells = torch.empty(n * 24, dtype=torch.uint8).pin_memory()
    import ctypes as C

    L = vtg.lib()
    torch.cuda.synchronize()
    e2e_steps = max(args.steps, 10)
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        cur = k & 1
        vtg.check(L.vtg_build(t.h, cur, C.c_void_p(pinned[cur].data_ptr()), W, vtg.HOST, None), "vtg_build")
        vtg.check(L.vtg_cells(t.h, cur ^ 1, cur, C.c_void_p(host_cells.data_ptr()), None, vtg.HOST, None), "vtg_cells")
        ctx.sync(10000)
    e2e_s = time.perf_counter() - t0
    e2e = {"value": n * e2e_steps / e2e_s, "unit": "cells/s", "h2d_bytes_per_step": W * H,
           "d2h_bytes_per_step": n * 24, "ms_per_step": 1e3 * e2e_s / e2e_steps}

    # the cells of one step, for the algorithmic FLOP count
    t.build(0, dframes[0].data_ptr(), W, where=vtg.DEVICE)
    t.build(1, dframes[1].data_ptr(), W, where=vtg.DEVICE)
    cells, lk = t.cells(0, 1)
    flops = lk_flops(lk, LEVELS)
    pk = peaks()
    sm_max = pk.get("sm_max_mhz", 2070.0)
    fp32_peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12
    lk_avg_s = float(lk_ms.mean()) / 1e3
    achieved = flops / lk_avg_s / 1e12
    roofline = {"kernel": "lk_cells_kernel", "bound": "fp32", "achieved": achieved, "peak": fp32_peak,
                "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                "peak_source": "nominal FP32 CUDA-core rate (152 SMs x 128 lanes x 2) at the measured max SM clock; "
                               "MEASURED_PEAKS.json holds no FP32 figure",
                "algorithmic_flop_per_launch": flops, "launch_ms": float(lk_ms.mean()), "traffic": None}
    pyr_ms = float((step_ms - lk_ms).mean())
    pyr_bytes = W * H + 4 * sum(a * b for a, b in [(1920, 1080), (960, 540), (480, 270), (240, 135)])
    roof_pyr = {"kernel": "pyr_reduce_kernel (3 launches)", "bound": "hbm", "achieved": pyr_bytes / (pyr_ms / 1e3) / 1e9,
                "peak": pk.get("hbm_gbs", 6800.0), "unit": "GB/s",
                "frac": pyr_bytes / (pyr_ms / 1e3) / 1e9 / pk.get("hbm_gbs", 6800.0),
                "algorithmic_bytes_per_step": pyr_bytes, "ms_per_step": pyr_ms,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in pk else "fallback"}
    t.close()
    ctx.close()
    line = {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded noise, blur 1.5, warp)",
            "config": workload("plain"), "p50_ms_per_pair": float(np.percentile(step_ms, 50)),
            "p99_ms_per_pair": float(np.percentile(step_ms, 99)), "e2e": e2e, "roofline": roofline,
            "roofline_pyramid": roof_pyr, "gpu_launches": args.steps * LEVELS, "clocks": clk.summary(),
            "wall_s": wall}
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(cells_sample=4050, frames=(f0, f1))
    return line if rank == 0 else None


def cpu_baseline(cells_sample: int, frames, threads: int | None = None) -> dict:
    """The oracle's FP64 restatement of the reference's path on the host cores: the pyramid of one frame and LK with
    forward-backward at the first `cells_sample` cells of the 16,200, repeated to at least 10 s."""
    sys.path.insert(0, ORACLE)
    import oracle as O

    threads = threads or os.cpu_count() or 1
    f0, f1 = frames
    xs, ys = O.cell_centres(W, H, CELL_W, CELL_H)
    xs, ys = xs[:cells_sample], ys[:cells_sample]
    cfg = O.lk_cfg()
    P0 = O.pyramid(f0, LEVELS)
    done, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < 10.0:
        P1 = O.pyramid(f1, LEVELS)
        O.lk_points(P0, P1, LEVELS - 1, cfg, xs, ys, max_fb=0.5, mode=O.F64, threads=threads)
        done += len(xs)
    dt = time.perf_counter() - t0
    import platform

    return {"value": done / dt, "unit": "cells/s", "cores": threads, "kind": "port",
            "sample": "pyramid + %d of 16,200 cells per repetition, FP64 oracle form, %d reps in %.1f s on %s" % (
                cells_sample, done // cells_sample, dt, platform.machine())}


def run_reference(args) -> dict | None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    sys.path.insert(0, ORACLE)
    import oracle as O
    import vtg_synth as S

    threads = os.cpu_count() or 1
    f0, f1, _, _ = S.warp_pair(W, H, S.seeded_shift(2, 0), 0.5, seed=2)
    xs, ys = O.cell_centres(W, H, CELL_W, CELL_H)
    sample = 2025  # one eighth of the grid, every 8th cell
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
    value = sample * args.steps / total
    import platform

    cb = {"value": value, "unit": "cells/s", "cores": threads, "kind": "port",
          "sample": "per step: the new frame's pyramid and every 8th cell (2,025 of 16,200), FP64 oracle form, %s" %
                    platform.machine()}
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded noise, blur 1.5, warp)", "config": workload("cpu"), "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="plain", choices=["plain"])
    ap.add_argument("--skip-e2e", action="store_true", help="time the kernels only (for profiling)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    line = run_reference(args) if args.impl == "reference" else run_ours(args)
    if line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
