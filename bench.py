"""Benchmark of the GB300 grid Morse-Smale path (one JSON line on rank 0).

Workload: the 4096x4096 float32 field of 512 Gaussian bumps quantised to
1/256 of its range (seed 1).  A step is one pass of the device pipeline over
that grid.  ``value`` is Mvertices/s with the heights already in HBM; ``e2e``
is the same metric through the public API with host (pinned) heights copied
in and the complex copied out every step.  ``--impl reference`` times the CPU
restatement of the reference path (the oracle) on the host cores instead.

Multi-GPU: the path does not shard (replicas only): every rank processes its
own grid, value = all vertices processed / max-over-ranks time.
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

METRIC = "Mvert/s at 4096^2 (% HBM roofline)"
WORKLOAD = ("bumps4096q: 4096x4096 float32, 512 Gaussian bumps (sigma U(4,64)) quantised to 1/256 of the range, "
            "seed 1; device pipeline: gradient, critical-cell collation, owner labels, connectivity")
STAGE_BYTES = {  # algorithmic bytes per vertex of each stage
    "gradient": 8.0,        # 4 B height read + 4 B gradient codes written
    "labels_arcs": 20.0,    # 4 B gradient codes read + 16 B owner labels written (+12 B/cp, 8 B/arc)
}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples (SM clock, reasons) during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_sample_field(field: np.ndarray, n: int) -> np.ndarray:
    return np.ascontiguousarray(field[:n, :n])


def cpu_baseline(field: np.ndarray, side: int = 1024):
    """The oracle (single thread) on a window of the same field, stages matching the device pipeline."""
    from oracle import oracle as O
    O.build()
    win = cpu_sample_field(field, side)
    t0 = time.perf_counter()
    P = O.Pipeline(win, levels=0, tresh=0.0)
    wall = time.perf_counter() - t0
    t = P.times_ms()
    secs = t["build"] / 1e3
    return {"value": round(win.size / secs / 1e6, 3), "unit": "Mvert/s", "cores": 1, "kind": "port",
            "sample": f"{side}x{side} window of the same field, oracle stages work+writeout_connectivity "
                      f"({secs:.2f} s; whole oracle run {wall:.2f} s)"}


def run_reference(args):
    """--impl reference: the oracle on the host cores (all threads via processes)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from mscomplex_gb300 import synth
    from oracle import oracle as O
    O.build()
    field = synth.bumps4096q()
    cores = os.cpu_count() or 1
    side = 512
    # windows of the same field, one per core, every step
    nwin = (field.shape[0] // side) * (field.shape[1] // side)
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_ref_init) as pool:
        for _ in range(args.warmup):
            pool.map(_ref_job, [(field, side, i % nwin) for i in range(cores)])
        t0 = time.perf_counter()
        verts = 0
        for s in range(args.steps):
            res = pool.map(_ref_job, [(field, side, (s * cores + i) % nwin) for i in range(cores)])
            verts += sum(res)
        dt = time.perf_counter() - t0
    value = verts / dt / 1e6
    line = {"metric": METRIC, "value": round(value, 3), "unit": "Mvert/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / max(1, args.steps), 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "sample": f"{cores} windows of {side}x{side} per step"},
            "cpu_baseline": {"value": round(value, 3), "unit": "Mvert/s", "cores": cores, "kind": "port",
                             "sample": f"{cores} processes, each the oracle (work+writeout_connectivity+discs) on a "
                                       f"{side}x{side} window of the field"},
            "e2e": {"value": round(value, 3), "unit": "Mvert/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _ref_init():
    sys.path.insert(0, ROOT)


def _ref_job(a):
    field, side, i = a
    from oracle import oracle as O
    nx = field.shape[1] // side
    y0, x0 = (i // nx) * side, (i % nx) * side
    win = np.ascontiguousarray(field[y0:y0 + side, x0:x0 + side])
    O.Pipeline(win, levels=0, tresh=0.0)
    return win.size


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import torch.distributed as dist

    import mscomplex_gb300 as M
    from mscomplex_gb300 import synth
    from mscomplex_gb300._native import kernel_launches

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    field = synth.bumps4096q()
    ny, nx = field.shape
    nverts = field.size
    rect = (0, 0, 2 * (nx - 1), 2 * (ny - 1))
    ctx = M.default_context(local)
    ctx.set_timing(True)
    dev = torch.from_numpy(field).cuda()
    ds = M.GridDataset(rect, rect, ctx=ctx)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > L2 (129 MB)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    def step():
        ds.init(dev, stream=sh)
        ds.work(stream=sh)
        return ds.writeout_connectivity(stream=sh)

    for _ in range(max(3, args.warmup)):
        msc = step()
    torch.cuda.synchronize()
    ncp, nasc, ndes = msc.sizes()[:3]

    # ---- device-resident timed region ----
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    launches0 = kernel_launches()
    times, stages = [], {k: [] for k in M.GridDataset.STAGES}
    for _ in range(args.steps):
        flush.fill_(1.0)  # evict L2 between steps (outside the timed interval)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        msc = step()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
        for k, v in ds.stage_times().items():
            stages[k].append(v)
    torch.cuda.synchronize()
    launches = kernel_launches() - launches0
    barrier()
    clk = clocks.stop()
    total_ms = sum(times)
    if world > 1:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = nverts * args.steps * world / (total_ms / 1e3) / 1e6

    # roofline of the dominant kernel (median stage time, live CUDA events)
    med = {k: statistics.median(v) for k, v in stages.items()}
    dom = max(STAGE_BYTES, key=lambda k: med[k])
    extra = 12.0 * ncp + 8.0 * (nasc + ndes) if dom == "labels_arcs" else 0.0
    alg_bytes = STAGE_BYTES[dom] * nverts + extra
    peak, peak_kind = peaks()
    achieved = alg_bytes / (med[dom] / 1e3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        traffic = json.load(open(tp)).get(f"{dom}:bumps4096q")
    pipe_bytes = 24.0 * nverts + 12.0 * ncp + 8.0 * (nasc + ndes)

    # ---- end to end through the public API (pinned host heights in, complex out) ----
    host = torch.from_numpy(field).pin_memory()
    h2d = host.numel() * 4
    d2h = 0
    barrier()
    e2e_times = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        s0 = time.perf_counter()
        d = host.to("cuda", non_blocking=True)
        ds.init(d, stream=sh)
        ds.work(stream=sh)
        out = ds.writeout_connectivity(stream=sh).export()
        e2e_times.append(time.perf_counter() - s0)
        d2h = sum(v.nbytes for v in out.values())
    e2e_total = sum(e2e_times)
    if world > 1:
        t = torch.tensor([e2e_total], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_total = float(t.item())
    e2e_value = nverts * args.steps * world / e2e_total / 1e6

    line = None
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mvert/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "grid": [nx, ny], "levels": 0, "critical_points": ncp,
                       "arcs": [nasc, ndes], "l2": "flushed between steps (256 MB write)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "stages_ms": {k: round(v, 4) for k, v in med.items()},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "alg_bytes_per_launch": int(alg_bytes), "traffic": traffic},
            "pipeline_roofline": {"alg_bytes": int(pipe_bytes),
                                  "frac": round(pipe_bytes / (total_ms / args.steps / 1e3) / 1e9 / peak, 4)},
            "e2e": {"value": round(e2e_value, 3), "unit": "Mvert/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "clocks": clk,
        }
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(field)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
