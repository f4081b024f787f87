"""Benchmark of the GB300 grid Morse-Smale path (one JSON line on rank 0).

Workload: the 4096x4096 float32 field of 512 Gaussian bumps quantised to
1/256 of its range (seed 1).  A step is one pass of the device path over that
grid: gradient, critical-cell collation, owner labels, connectivity (the
complex) and the ascending/descending manifold discs of every critical point.
``value`` is Mvertices/s with the heights already in HBM; ``e2e`` is the same
step through the public API with host (pinned) heights copied in and the
complex with its discs copied out every step.

Persistence cancellation at 1% of the range is not inside the timed step: on
this field the reference's tie order (its heap) needs ~5.9e9 dependent heap
operations, which the device replays exactly but sequentially.  It is
measured beside the step ("simplify": device replay operations per second
under an operation budget, and the whole-field estimate from the operation
count).

``--impl reference`` times the CPU restatement of the reference path (the
oracle) on the host cores instead.  Multi-GPU: the path does not shard
(replicas only): every rank processes its own grid, value = all vertices
processed / max-over-ranks time.
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
            "seed 1; step = gradient, critical-cell collation, owner labels, connectivity, manifold discs; "
            "persistence cancellation at 1% measured separately (see simplify)")
SIMPLIFY_TRESH = 0.01
# heap pushes + pops of the reference's simplification of this field at 1%,
# counted by the oracle (2.956808816e9 pushes, 2.954259461e9 pops)
SIMPLIFY_HEAP_OPS = 2956808816 + 2954259461
# The kernels of the step that the launch list ranks highest, each timed live
# with its own CUDA events, with their algorithmic bytes (outputs and the
# height input only; intermediate structures are not counted):
#   (per vertex, per critical point, per arc, per saddle disc cell of the asc / des kind)
KERNEL_BYTES = {
    "gradient": (8.0, 0, 0, 0, 0),        # k_gradient: 4 B height read + 4 B gradient codes (1 B per cell)
    "labels_arcs": (16.0, 12, 8, 0, 0),   # k_labels: 16 B owner labels (4 B per cell), cp records, arcs
    "disc_hops": (4.0, 0, 0, 0, 0),       # k_disc_hops: reads the gradient codes (4 B/vertex); writes only the
                                          # hop structure and successor words (intermediates, not counted)
    # the saddle discs of one kind: k_win_place (and the level-0 items and the discs of saddles with many
    # chains); 4 B per saddle disc cell written
    "seg_place_asc": (0.0, 0, 0, 4, 0),
    "seg_place_des": (0.0, 0, 0, 0, 4),
}
KERNEL_NAMES = {"gradient": "k_gradient", "labels_arcs": "k_labels", "disc_hops": "k_disc_hops",
                "seg_place_asc": "k_win_place", "seg_place_des": "k_win_place"}
TRAFFIC_KEYS = {"gradient": "k_gradient", "labels_arcs": "k_labels", "disc_hops": "k_disc_hops",
                "seg_place_asc": "k_win_place:asc", "seg_place_des": "k_win_place:des"}
# The whole step: 24 B/vertex (height, gradient, owner labels) + 12 B/cp + 8 B/arc + 4 B per disc cell written.
PIPE_BYTES = (24.0, 12, 8, 4)


def stage_bytes(stage, nverts, ncp, narcs, ndisc, sdisc=(0, 0)):
    if stage == "pipeline":
        v, c, a, d = PIPE_BYTES
        return v * nverts + c * ncp + a * narcs + d * ndisc
    v, c, a, sa, sd = KERNEL_BYTES.get(stage, (0, 0, 0, 0, 0))
    return v * nverts + c * ncp + a * narcs + sa * sdisc[0] + sd * sdisc[1]


def saddle_disc_cells(ex: dict):
    """Cells of the saddles' asc and des discs in an exported complex."""
    c = ex["cellid"].astype(np.int64)
    sad = ((c[:, 0] & 1) + (c[:, 1] & 1)) == 1
    return (int(np.diff(ex["adisc_off"].astype(np.int64))[sad].sum()),
            int(np.diff(ex["ddisc_off"].astype(np.int64))[sad].sum()))


def simplify_rate(M, field: np.ndarray, torch, side: int = 1024):
    """The exact device replay of simplify_un_simplify at 1% on the field's
    side x side corner window, run to completion: its time and heap
    operations per second.  The same window is what the oracle's rate is
    timed on (cpu_simplify_rate), so the two rates compare like for like."""
    win = cpu_sample_field(field, side)
    r = (0, 0, 2 * (side - 1), 2 * (side - 1))
    ds = M.GridDataset(r, r).init(win).work()
    m = ds.writeout_connectivity()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    try:
        m.simplify_un_simplify(SIMPLIFY_TRESH)
        done = True
    except M.DmscError:
        done = False
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    st = m.simplify_stats()
    heap_ops = st["pops"] + st["pushes"]
    rate = heap_ops / secs if secs > 0 else None
    return {"threshold": SIMPLIFY_TRESH, "window": f"{side}x{side} corner of the field", "completed": done,
            "heap_ops": int(heap_ops), "cancellations": st["cancels"], "s": round(secs, 3),
            "heap_ops_per_s": round(rate, 1) if rate else None, "field_heap_ops": SIMPLIFY_HEAP_OPS,
            "field_est_s": round(SIMPLIFY_HEAP_OPS / rate, 1) if rate else None,
            "note": "one sequential replay of the reference's heap (its tie order decides the result); "
                    "not part of the timed step"}


def cpu_simplify_rate(field: np.ndarray, side: int = 1024):
    """The oracle's simplify_un_simplify (one thread, libstdc++ heap) at 1% on
    the same window, run to completion on the host: heap operations per
    second (the time of the run with simplification minus the time without)."""
    from oracle import oracle as O
    O.build()
    win = cpu_sample_field(field, side)
    r = (0, 0, 2 * (side - 1), 2 * (side - 1))
    t0 = time.perf_counter()
    O.Dataset(win, r, r, tresh=0.0)
    t1 = time.perf_counter()
    O.simplify_stats()
    O.Dataset(win, r, r, tresh=SIMPLIFY_TRESH)
    t2 = time.perf_counter()
    st = O.simplify_stats()
    secs = max(1e-9, (t2 - t1) - (t1 - t0))
    ops = st["pushes"] + st["pops"]
    return {"cpu_heap_ops_per_s": round(ops / secs, 1), "cpu_s": round(secs, 3), "cpu_cores": 1,
            "cpu_field_est_s": round(SIMPLIFY_HEAP_OPS / (ops / secs), 1),
            "cpu_sample": f"{side}x{side} window of the field at 1% of its range: {ops} heap operations, "
                          f"{st['cancels']} cancellations, {secs:.2f} s"}


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


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """The maximum of x over all ranks (the job's time is its slowest rank's)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_value(units_per_rank: float, world: int, seconds: float) -> float:
    """Whole-job throughput of N replicas: all ranks' units over the slowest rank's time."""
    return units_per_rank * world / seconds


def gpu_local_cpus(device: int):
    """The host CPUs next to the GPU (sysfs local_cpulist of its PCI device),
    intersected with the CPUs this process may use; empty if unknown."""
    try:
        import torch
        pr = torch.cuda.get_device_properties(device)
        bus = "%04x:%02x:%02x.0" % (getattr(pr, "pci_domain_id", 0), pr.pci_bus_id, pr.pci_device_id)
        with open(f"/sys/bus/pci/devices/{bus}/local_cpulist") as fh:
            spec = fh.read().strip()
        cpus = set()
        for part in spec.split(","):
            if "-" in part:
                lo, hi = part.split("-")
                cpus.update(range(int(lo), int(hi) + 1))
            elif part:
                cpus.add(int(part))
        return sorted(cpus & os.sched_getaffinity(0))
    except Exception:
        return []


def host_link(torch, nbytes=800 << 20, reps=3):
    """Pinned host <-> device copy bandwidth (GB/s) of one large copy each way."""
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = {}
    for name, dst, src in (("d2h_gbs", h, d), ("h2d_gbs", d, h)):
        best = 0.0
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            dst.copy_(src, non_blocking=True)
            torch.cuda.synchronize()
            best = max(best, nbytes / (time.perf_counter() - t0) / 1e9)
        out[name] = round(best, 1)
    del h, d
    return out


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_sample_field(field: np.ndarray, n: int) -> np.ndarray:
    return np.ascontiguousarray(field[:n, :n])


def oracle_step(win: np.ndarray) -> float:
    """One step of the oracle on a window: init, work, writeout_connectivity and
    postMergeFillDiscs (the stages of the device step); returns seconds."""
    from oracle import oracle as O
    r = (0, 0, 2 * (win.shape[1] - 1), 2 * (win.shape[0] - 1))
    t0 = time.perf_counter()
    O.Dataset(win, r, r, tresh=0.0, fill_discs=True)
    return time.perf_counter() - t0


def cpu_baseline(field: np.ndarray, side: int = 1024):
    """The oracle (single thread) on a window of the same field, same stages as the device step."""
    from oracle import oracle as O
    O.build()
    win = cpu_sample_field(field, side)
    secs = oracle_step(win)
    return {"value": round(win.size / secs / 1e6, 3), "unit": "Mvert/s", "cores": 1, "kind": "port",
            "sample": f"{side}x{side} window of the same field, one oracle step (work, writeout_connectivity, "
                      f"postMergeFillDiscs) in {secs:.2f} s"}


BATCH_WORKLOAD = ("batch_fields: 1000 grids, sides log-uniform in [64, 2048], each a float32 sum of Gaussians "
                  "(count = area / 8192, sigma U(4, 32)), seed 3; work + writeout_connectivity + "
                  "simplify_un_simplify at 2% of each grid's range")


def bench_batched(M, torch, stream, sh, steps=2, warmup=1, count=1000):
    """Mixed-size batch: one batched pass over all grids versus one plain
    per-grid pass (dataset, work, writeout_connectivity, simplify per grid),
    both from heights resident in HBM; e2e batch from pinned host heights to
    every complex in pinned host memory.  Returns the JSON object."""
    from mscomplex_gb300 import synth
    fields = synth.batch_fields(count)
    packed, sizes = M.GridBatch.pack(fields)
    nverts = int(packed.size)
    dev = torch.from_numpy(packed).cuda()
    torch.cuda.synchronize()
    tresh = 0.02
    b = M.GridBatch()
    for _ in range(max(1, warmup)):
        b.run(packed=dev, sizes=sizes, tresh=tresh, stream=sh)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        b.run(packed=dev, sizes=sizes, tresh=tresh, stream=sh)
    e1.record(stream)
    e1.synchronize()
    batch_s = e0.elapsed_time(e1) / 1e3 / steps
    # plain: one grid at a time through the per-grid API
    offs = np.concatenate([[0], np.cumsum(sizes[0::2].astype(np.int64) * sizes[1::2])])
    views = [dev[offs[i]:offs[i + 1]].view(int(sizes[2 * i + 1]), int(sizes[2 * i])) for i in range(count)]
    def plain(check_idx=()):
        outs = {}
        for i, v in enumerate(views):
            r = (0, 0, 2 * (v.shape[1] - 1), 2 * (v.shape[0] - 1))
            ds = M.GridDataset(r, r).init(v, stream=sh).work(stream=sh)
            m = ds.writeout_connectivity(stream=sh)
            m.simplify_un_simplify(tresh, stream=sh)
            if i in check_idx:
                outs[i] = m.export()
        return outs
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ref = plain(check_idx=set(range(0, count, max(1, count // 16))))
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    keys = M.GridBatch.GRAPH_KEYS
    exact = all(all(np.array_equal(np.asarray(b.export(i)[k]).view(np.uint8), np.asarray(ref[i][k]).view(np.uint8))
                    for k in keys) for i in ref)
    # e2e: pinned host heights in, every complex out into pinned host memory
    host = torch.from_numpy(packed).pin_memory()
    ncp, na, nd = b.totals()
    pinned = {k: torch.empty(max(16, 4 * (m * 5 // 4 + 16)), dtype=torch.uint8).pin_memory().numpy()
              for k, m in (("cp_base", count + 1), ("asc_base", count + 1), ("des_base", count + 1), ("cellid", ncp),
                           ("fn", ncp), ("pair_idx", ncp), ("flags", ncp), ("asc_off", ncp + 1), ("asc", na),
                           ("des_off", ncp + 1), ("des", nd))}
    def e2e_pass():
        d = host.to("cuda", non_blocking=True)
        b.run(packed=d, sizes=sizes, tresh=tresh, stream=sh)
        return b.export_all(pinned)

    e2e_pass()  # untimed: the first copies into and out of freshly pinned buffers pay a one-time set-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d2h = 0
    for _ in range(steps):
        out = e2e_pass()
        d2h = sum(v.nbytes for v in out.values())
    e2e_s = (time.perf_counter() - t0) / steps
    st = [b.simplify_stats(i) for i in range(count)]
    tile_ms = b.tile_times()
    # the launch autotuner on the workload's own grids, then the batched pass again
    t0 = time.perf_counter()
    table = M.GridBatch.autotune(fields, repeats=2)
    tune_s = time.perf_counter() - t0
    bt = M.GridBatch()
    bt.run(packed=dev, sizes=sizes, tresh=tresh, stream=sh)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        bt.run(packed=dev, sizes=sizes, tresh=tresh, stream=sh)
    e1.record(stream)
    e1.synchronize()
    tuned_s = e0.elapsed_time(e1) / 1e3 / steps
    tuned_tile_ms = bt.tile_times()
    exact = exact and all(all(np.array_equal(np.asarray(bt.export(i)[k]).view(np.uint8),
                                             np.asarray(ref[i][k]).view(np.uint8)) for k in keys) for i in ref)
    M.GridBatch.autotune_reset()
    return {"workload": BATCH_WORKLOAD, "grids": count, "vertices": nverts, "critical_points": ncp,
            "batched_grids_per_s": round(count / batch_s, 2), "batched_mvert_per_s": round(nverts / batch_s / 1e6, 2),
            "batched_ms": round(batch_s * 1e3, 3), "plain_grids_per_s": round(count / plain_s, 2),
            "plain_ms": round(plain_s * 1e3, 3), "speedup_vs_plain": round(plain_s / batch_s, 2),
            "e2e_grids_per_s": round(count / e2e_s, 2), "e2e_h2d_bytes": int(packed.nbytes), "e2e_d2h_bytes": int(d2h),
            "bit_exact_vs_plain": bool(exact), "checked_grids": len(ref),
            "tile_kernels_ms": [round(v, 3) for v in tile_ms],
            "autotune": {"seconds": round(tune_s, 2), "per_class": {k: {"threads": v[0], "blocks_per_sm": v[1],
                                                                        "tile_us": v[2], "default_tile_us": v[3]}
                                                                    for k, v in table.items()},
                         "batched_grids_per_s": round(count / tuned_s, 2), "batched_ms": round(tuned_s * 1e3, 3),
                         "tile_kernels_ms": [round(v, 3) for v in tuned_tile_ms]},
            "max_simplify_pops": max(x["pops"] for x in st), "total_simplify_pops": sum(x["pops"] for x in st)}


SERVE_WORKLOAD = ("served: Poisson arrivals; sides 80% U(128,512), 18% U(1024,2048), 2% 4096; Gaussian sums "
                  "(10% quantised to 1/256 of the range); tresh U(0, 5%); arena 150 GB; seed 4")


def serve_requests(count: int, seed: int = 4):
    """The served request mix: (field, tresh) pairs."""
    from mscomplex_gb300 import synth
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        u = rng.random()
        side = int(rng.integers(128, 513)) if u < 0.8 else int(rng.integers(1024, 2049)) if u < 0.98 else 4096
        quant = 256 if rng.random() < 0.1 else 0
        reqs.append((synth.mixed_grid(side, seed * 7919 + i, quantize=quant), float(rng.uniform(0.0, 0.05))))
    return reqs


def bench_served(M, torch, count=300, rates=((None, 300), (200.0, 300), (40.0, 120), (20.0, 120), (10.0, 120)),
                 max_ops=2_000_000, lanes=4):
    """The request server under a Poisson stream (rate None = every request
    submitted at once, i.e. saturation; each rate with its number of
    requests, the first ones of the same mix) against plain
    one-request-at-a-time processing through the per-grid API.  Latency =
    submit -> result ready; grids_per_s counts completed requests only."""
    reqs = serve_requests(count)
    out = {"workload": SERVE_WORKLOAD, "requests": count, "max_ops_per_request": max_ops, "lanes": lanes, "runs": []}
    for rate, nreq in rates:
        rng = np.random.default_rng(11)
        gaps = np.zeros(nreq) if rate is None else rng.exponential(1.0 / rate, nreq)
        srv = M.GridServer(arena_bytes=150 << 30, lanes=lanes, max_batch=128, max_ops=max_ops)
        t0 = time.perf_counter()
        ids = []
        next_t = 0.0
        for (f, t), gap in zip(reqs[:nreq], gaps):
            next_t += gap
            while time.perf_counter() - t0 < next_t:
                time.sleep(0.0002)
            ids.append(srv.submit(f, t))
        lat, fails = [], 0
        for rid in ids:
            try:
                r = srv.result(rid)
                s0, _, d0 = r["times_ms"]
                lat.append(d0 - s0)
            except M.DmscError:
                fails += 1
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        lat = np.array(lat) if lat else np.zeros(1)
        out["runs"].append({"rate_per_s": rate if rate is not None else "saturation", "requests": nreq,
                            "completed": nreq - fails, "failed": fails, "failed_frac": round(fails / nreq, 4),
                            "grids_per_s": round((nreq - fails) / wall, 2),
                            "p50_ms": round(float(np.percentile(lat, 50)), 2),
                            "p99_ms": round(float(np.percentile(lat, 99)), 2), "batches": st["batches"]})
    # plain: one request at a time, each through dataset / writeout / simplify / export;
    # all submitted at t0 like the saturation run, so latency includes waiting
    t0 = time.perf_counter()
    lat, svc, fails = [], [], 0
    for f, t in reqs:
        s0 = time.perf_counter()
        try:
            r = (0, 0, 2 * (f.shape[1] - 1), 2 * (f.shape[0] - 1))
            m = M.GridDataset(r, r).init(f).work().writeout_connectivity()
            if t > 0:
                m.simplify_un_simplify(t, max_ops=max_ops)
            m.export()
        except M.DmscError:
            fails += 1
            continue
        now = time.perf_counter()
        svc.append((now - s0) * 1e3)
        lat.append((now - t0) * 1e3)
    wall = time.perf_counter() - t0
    lat, svc = np.array(lat), np.array(svc)
    out["plain"] = {"grids_per_s": round((count - fails) / wall, 2), "completed": count - fails, "failed": fails,
                    "p50_ms": round(float(np.percentile(lat, 50)), 2),
                    "p99_ms": round(float(np.percentile(lat, 99)), 2),
                    "service_p50_ms": round(float(np.percentile(svc, 50)), 2),
                    "service_p99_ms": round(float(np.percentile(svc, 99)), 2),
                    "note": "sequential, all submitted at once: latency = completion time since submission"}
    sat = out["runs"][0]["grids_per_s"]
    out["speedup_vs_plain"] = round(sat / out["plain"]["grids_per_s"], 2)
    return out


PIPE_WORKLOAD = ("noise16384: 16384x16384 float32 i.i.d. U[0,1), seed 2; 8 levels of binary splits alternating y and x "
                 "(256 blocks of 1024x1024 with a one-vertex halo); one complex per block, merge up to the root, "
                 "tresh 0, merge down, manifold discs of every block")


def bench_pipeline(M, torch, n=16384, levels=8, runs=2, cpu_side=1024):
    """The whole piece pipeline on the white-noise field (heights resident in
    HBM), wall clock per run; stage times from the library."""
    from mscomplex_gb300 import synth
    f = torch.from_numpy(synth.noise(n, seed=2)).cuda()
    torch.cuda.synchronize()
    walls, last = [], None
    for r in range(runs + 1):  # the first run is warm-up
        t0 = time.perf_counter()
        p = M.GridDataManager(f, levels=levels, tresh=0.0, split2d=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if r:
            walls.append(dt)
        last = (p.stage_times(), p.merge_seq_times(), p.piece(2 * p.num_pieces - 2).sizes())
        del p
    wall = statistics.median(walls)
    stages, seq, root = last
    out = {"workload": PIPE_WORKLOAD, "Mvert_per_s": round(n * n / wall / 1e6, 2), "s_per_run": round(wall, 3),
           "runs": runs, "stages_ms": {k: round(v, 1) for k, v in stages.items()},
           "boundary_steps_ms": {k: round(v, 1) for k, v in seq.items()},
           "root_complex": {"critical_points": root[0], "asc": root[1], "des": root[2]}}
    if cpu_side:
        # the oracle's whole pipeline (one thread) on a smaller field of the same kind, 2 levels of splits
        from oracle import oracle as O
        O.build()
        g = synth.noise(cpu_side, seed=2)
        t0 = time.perf_counter()
        O.Pipeline(g, levels=2, tresh=0.0, split2d=True)
        secs = time.perf_counter() - t0
        out["cpu_oracle"] = {"value": round(g.size / secs / 1e6, 3), "unit": "Mvert/s", "cores": 1, "kind": "port",
                             "sample": f"{cpu_side}x{cpu_side} white noise (seed 2), 4 blocks of {cpu_side // 2}^2, "
                                       f"the oracle's whole pipeline in {secs:.1f} s"}
    return out


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
    nx = field.shape[1] // side

    def window(i):
        y0, x0 = (i // nx) * side, (i % nx) * side
        return np.ascontiguousarray(field[y0:y0 + side, x0:x0 + side])

    with ctx.Pool(cores, initializer=_ref_init) as pool:
        for _ in range(args.warmup):
            pool.map(_ref_job, [window(i % nwin) for i in range(cores)])
        t0 = time.perf_counter()
        verts = 0
        for s in range(args.steps):
            res = pool.map(_ref_job, [window((s * cores + i) % nwin) for i in range(cores)])
            verts += sum(res)
        dt = time.perf_counter() - t0
    value = verts / dt / 1e6
    line = {"metric": METRIC, "value": round(value, 3), "unit": "Mvert/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / max(1, args.steps), 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "sample": f"{cores} windows of {side}x{side} per step"},
            "cpu_baseline": {"value": round(value, 3), "unit": "Mvert/s", "cores": cores, "kind": "port",
                             "sample": f"{cores} processes, each one oracle step (work, writeout_connectivity, postMergeFillDiscs) on a "
                                       f"{side}x{side} window of the field"},
            "e2e": {"value": round(value, 3), "unit": "Mvert/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _ref_init():
    sys.path.insert(0, ROOT)


def _ref_job(win):
    oracle_step(win)
    return win.size


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="leave out the mixed-size batch measurement")
    ap.add_argument("--no-pipeline", action="store_true", help="leave out the 16384^2 piece-pipeline measurement")
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
    # host threads and pinned buffers on the CPUs next to the GPU (first touch
    # places pinned pages on the calling thread's node)
    local_cpus = gpu_local_cpus(local)
    if local_cpus:
        os.sched_setaffinity(0, local_cpus)
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
    # one non-default stream for everything: the library's kernels, the L2
    # flush, host copies and the timing events are ordered on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream

    held = {}  # one complex per loop, overwritten in place every step

    def step(slot="dev"):
        ds.init(dev, stream=sh)
        ds.work(stream=sh)
        m = held[slot] = ds.writeout_connectivity(held.get(slot), stream=sh)
        ds.post_merge_fill_discs(m, stream=sh)
        return m

    for _ in range(max(3, args.warmup)):
        msc = step()
    torch.cuda.synchronize()
    ncp, nasc, ndes, nadisc, nddisc = msc.sizes()
    sdisc = saddle_disc_cells(msc.export())

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
        for k, v in ds.stage_times(with_discs=True).items():
            stages[k].append(v)
    torch.cuda.synchronize()
    launches = kernel_launches() - launches0
    barrier()
    clk = clocks.stop()
    total_ms = max_over_ranks(sum(times), world)
    value = replicas_value(nverts * args.steps, world, total_ms / 1e3) / 1e6

    # roofline of the dominant kernel: the longest of the live-timed kernels
    # (median over the steps), its algorithmic bytes over that time
    med = {k: statistics.median(v) for k, v in stages.items()}
    dom = max(KERNEL_BYTES, key=lambda k: med[k])
    alg_bytes = stage_bytes(dom, nverts, ncp, nasc + ndes, nadisc + nddisc, sdisc)
    peak, peak_kind = peaks()
    achieved = alg_bytes / (med[dom] / 1e3) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        traffic = json.load(open(tp)).get(f"{TRAFFIC_KEYS[dom]}:bumps4096q")
    kernels = {k: {"kernel": KERNEL_NAMES[k], "ms": round(med[k], 4),
                   "alg_bytes": int(stage_bytes(k, nverts, ncp, nasc + ndes, nadisc + nddisc, sdisc)),
                   "frac": round(stage_bytes(k, nverts, ncp, nasc + ndes, nadisc + nddisc, sdisc)
                                 / (med[k] / 1e3) / 1e9 / peak, 4)} for k in KERNEL_BYTES}
    pipe_bytes = stage_bytes("pipeline", nverts, ncp, nasc + ndes, nadisc + nddisc)

    # ---- persistence cancellation at 1%: device replay rate under an operation budget ----
    simp = simplify_rate(M, field, torch)

    # ---- end to end through the public API (pinned host heights in, complex out) ----
    # Every step copies its heights in from pinned host memory and its whole
    # complex with discs out into pinned host memory.  The copies overlap the
    # computation of the neighbouring steps: step i+1's heights come in on an
    # input stream and step i's complex goes out on an output stream while
    # step i computes / step i+1 computes.  Two device height buffers, two
    # complexes and two sets of host buffers alternate; a buffer or complex is
    # rewritten only after what read it last is done.  The K steps are timed
    # as one span, from the first input copy to the last result copy.
    link = host_link(torch)
    host = torch.from_numpy(field).pin_memory()
    in_stream = torch.cuda.Stream()
    dbuf, used, ready = [torch.empty_like(dev), torch.empty_like(dev)], [None, None], [None, None]

    def fetch(j):  # step j's heights into device buffer j % 2, on the input stream
        b = j & 1
        if used[b] is not None:
            in_stream.wait_event(used[b])
        with torch.cuda.stream(in_stream):
            dbuf[b].copy_(host, non_blocking=True)
        ready[b] = in_stream.record_event()

    def pinned_set():  # sized from the warm-up result, 25% headroom
        out = {}
        for k, (shape, dt) in msc.export_shapes().items():
            n = int(np.prod(shape)) * 5 // 4 + 16
            out[k] = torch.empty(n * np.dtype(dt).itemsize, dtype=torch.uint8).pin_memory().numpy()
        return out

    pinned = [pinned_set(), pinned_set()]
    copy_stream = torch.cuda.Stream()
    slots, freed = [None, None], [None, None]
    h2d = host.numel() * 4

    def e2e_steps(nsteps):
        fetch(0)
        out = None
        for i in range(nsteps):
            k = i & 1
            flush.fill_(1.0)
            stream.wait_event(ready[k])
            if i + 1 < nsteps:
                fetch(i + 1)
            ds.init(dbuf[k], stream=sh)
            ds.work(stream=sh)
            used[k] = stream.record_event()  # the heights are read by the gradient and the labels only
            if freed[k] is not None:
                stream.wait_event(freed[k])
            m = slots[k] = ds.writeout_connectivity(slots[k], stream=sh)
            ds.post_merge_fill_discs(m, stream=sh)
            copy_stream.wait_event(stream.record_event())
            out = m.export(pinned[k], stream=copy_stream.cuda_stream, wait=False)
            freed[k] = copy_stream.record_event()
        return out

    # untimed warm-up of the same loop: the first host-to-device and
    # device-to-host copies of a process pay one-time set-up costs (about
    # 250 ms on the GB300's host link)
    e2e_steps(max(3, args.warmup))
    barrier()
    torch.cuda.synchronize()
    s0 = time.perf_counter()
    out = e2e_steps(args.steps)
    torch.cuda.synchronize()
    e2e_total = max_over_ranks(time.perf_counter() - s0, world)
    d2h = sum(v.nbytes for v in out.values())
    e2e_value = replicas_value(nverts * args.steps, world, e2e_total) / 1e6
    ref = msc.export()  # the same heights through the device-resident step
    if any(not np.array_equal(ref[k], out[k]) for k in ref):
        raise RuntimeError("the end-to-end complex differs from the device-resident one")

    line = None
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mvert/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "grid": [nx, ny], "levels": 0, "critical_points": ncp,
                       "arcs": [nasc, ndes], "disc_cells": [nadisc, nddisc],
                       "saddle_disc_cells": list(sdisc),
                       "simplification": "excluded from the step; measured in simplify",
                       "l2": "flushed between steps (256 MB write)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "stages_ms": {k: round(v, 4) for k, v in med.items()},
            "roofline": {"bound": "hbm", "kernel": KERNEL_NAMES[dom], "stage": dom, "achieved": round(achieved, 1),
                         "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "alg_bytes_per_launch": int(alg_bytes), "traffic": traffic},
            "kernels": kernels,
            "pipeline_roofline": {"alg_bytes": int(pipe_bytes),
                                  "frac": round(pipe_bytes / (total_ms / args.steps / 1e3) / 1e9 / peak, 4)},
            "simplify": simp,
            "e2e": {"value": round(e2e_value, 3), "unit": "Mvert/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "host_link": dict(link, cpus=len(local_cpus) or None),
            "gpu_launches": int(launches),
            "clocks": clk,
        }
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(field)
            line["simplify"].update(cpu_simplify_rate(field))
        if world == 1 and not args.no_batch:
            line["batched"] = bench_batched(M, torch, stream, sh)
            line["served"] = bench_served(M, torch)
        if world == 1 and not args.no_pipeline:
            line["pipeline"] = bench_pipeline(M, torch, cpu_side=0 if args.no_cpu_baseline else 1024)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
