"""Benchmark: coupe Rcb on one GB300 (and N replicas under torchrun).

Workload (one "step"): Rcb of 16,777,216 3D points (a mixture of 32 Gaussians)
with int64 weights U{1..100} into 1024 parts (iter_count 10, tolerance 0.01).
Inputs are 537 MB per step (larger than the 129 MB L2), so no L2 flush is
needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload gauss16M|uniform1M|planes67M|batched4096|hexrib134M]

`value`   device-resident throughput (inputs in HBM before the timed region),
          Mpoints/s, of the headline precision mode.
`e2e`     the same metric through the C ABI (coupe_gpu_rcb) with pinned host
          buffers: host->device copies and the part-id read-back are inside.
`roofline` the kernel with the largest share of device time, its algorithmic
          bytes per launch over its CUDA-event duration, against the measured
          HBM copy bandwidth.
`cpu_baseline` the CPU restatement of coupe's Rcb (OpenMP, all host cores).
--impl reference times that CPU restatement alone (the reference itself is
Rust and cannot be built here).

The other workloads (--workload) print one line of the same form for plain
Rcb of 1M 2D points (8 parts, unit weights; inputs below L2 size, so L2 is
flushed before each timed step), the precision form on 67M points (4096
parts, f64 weights), the batched form (4096 sets, ~2e8 points) and Rib on a
512^3 hex mesh (134M points); with --impl reference, the CPU restatement's
line for the same workload.
"""
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

METRIC = "RCB Mpoints/s, 16M 3D pts→1024 parts: FP32-key+FP64-band vs plain FP64 on GB300"
UNIT = "Mpoints/s"
L2_FLUSH_BELOW = 256 << 20  # inputs below this size: L2 is flushed before each timed step


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--points", type=int, default=16_777_216)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--workload", default="gauss16M", choices=["gauss16M", "uniform1M", "planes67M", "batched4096", "hexrib134M"])
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for i, nm in enumerate(names):
                    if r[5 + i].lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(pts, w, cfg, budget_s=20.0):
    """The oracle (OpenMP restatement of coupe's rayon Rcb) on all host cores,
    on the full workload, repeated while the time budget lasts."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    times, ids = [], None
    t_end = time.perf_counter() + budget_s
    while True:
        t0 = time.perf_counter()
        ids, _ = oracle.rcb(pts, w, cfg["iter_count"], cfg["tolerance"], threads=0)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() + times[-1] > t_end or len(times) >= 5:
            break
    t = statistics.median(times)
    cores = os.cpu_count()
    return {"value": len(pts) / t / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "full workload (%d points), %d runs, median %.3f s; OpenMP restatement of coupe "
                      "Rcb (reference is Rust, not buildable here)" % (len(pts), len(times), t)}, ids


def _headline_config(cfg, n, input_bytes):
    """The workload description both arms print (identical dicts)."""
    return {"workload": cfg["name"], "points": n, "dim": 3, "parts": 1 << cfg["iter_count"],
            "iter_count": cfg["iter_count"], "tolerance": cfg["tolerance"], "weights": "int64 U{1..100}",
            "l2": "inputs larger than L2 (%d MB per step), no flush" % (input_bytes >> 20)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from coupe_gb300 import workloads
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    pts, w, cfg = workloads.gaussian_mixture3d(n=args.points)
    n = len(pts)
    # size each step so that the whole run ends within a few minutes
    t0 = time.perf_counter()
    oracle.rcb(pts, w, cfg["iter_count"], cfg["tolerance"], threads=0)
    t_full = time.perf_counter() - t0
    sample = n
    if t_full * (args.steps + args.warmup) > 150.0:
        sample = max(1 << 16, int(n * 150.0 / (t_full * (args.steps + args.warmup))))
    ps, ws = pts[:sample], w[:sample]
    for _ in range(max(0, args.warmup - 1)):
        oracle.rcb(ps, ws, cfg["iter_count"], cfg["tolerance"], threads=0)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.rcb(ps, ws, cfg["iter_count"], cfg["tolerance"], threads=0)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    value = sample / (ms / 1e3) / 1e6
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": _headline_config(cfg, n, pts.nbytes + w.nbytes),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d of %d points per step (first points of the seeded workload); OpenMP "
                                   "restatement of coupe Rcb on all host cores" % (sample, n)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args) if args.workload == "gauss16M" else run_reference_workload(args)
    if args.workload != "gauss16M":
        return run_workload(args)
    import torch
    import torch.distributed as dist
    import coupe_gb300 as coupe
    from coupe_gb300 import workloads

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    coupe.lib()

    pts_h, w_h, cfg = workloads.gaussian_mixture3d(n=args.points, seed=rank)
    n = len(pts_h)
    iters, tol = cfg["iter_count"], cfg["tolerance"]
    pts = torch.from_numpy(pts_h).to(dev)
    w = torch.from_numpy(w_h).to(dev)
    part = torch.empty(n, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    modes = ["ref32", "f64"]
    if coupe.MODES.get("f32key_f64band") is not None and _mode_available(coupe, pts, w, part):
        modes.append("f32key_f64band")
    headline = "f32key_f64band" if "f32key_f64band" in modes else "ref32"

    results, launches, ids_by_mode = {}, {}, {}
    clocks = None
    for mode in modes:
        for _ in range(args.warmup):
            coupe.rcb_device(part, pts, w, iters, tol, mode=mode)
        barrier()
        if mode == headline:
            clocks = Clocks(local).__enter__()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        nl = 0
        ev0.record(stream)
        for _ in range(args.steps):
            coupe.rcb_device(part, pts, w, iters, tol, mode=mode)
            nl += coupe.last_stats()["kernel_launches"]
        ev1.record(stream)
        barrier()
        if mode == headline:
            clocks.__exit__()
        ms = ev0.elapsed_time(ev1) / args.steps
        if world > 1:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        results[mode] = ms
        launches[mode] = nl
        ids_by_mode[mode] = part.cpu().numpy().view(np.uint64).copy()
    stats = coupe.last_stats()

    # live roofline: per-kernel CUDA-event times over K more steps (every
    # mode, for the per-kernel comparison; the headline mode's for the roofline)
    by_mode = {}
    for mode in modes:
        coupe.profile(True)
        for _ in range(args.steps):
            coupe.rcb_device(part, pts, w, iters, tol, mode=mode)
        torch.cuda.synchronize()
        by_mode[mode] = coupe.profile_read()
        coupe.profile(False)
    prof = by_mode[headline]
    total_ms = sum(v["ms"] for v in prof.values()) or 1.0
    top = max(prof.items(), key=lambda kv: kv[1]["ms"])
    peak, peak_kind = measured_peak()
    achieved = top[1]["bytes"] / (top[1]["ms"] / 1e3) / 1e9
    traffic = _traffic_per_launch(top[0], headline, "gauss16M")
    roofline = {"bound": "hbm", "kernel": top[0], "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "traffic": traffic, "algorithmic_bytes_per_launch": top[1]["bytes"] // max(1, top[1]["launches"]),
                "launches": top[1]["launches"], "share": round(top[1]["ms"] / total_ms, 3),
                "kernels": {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                                "share": round(v["ms"] / total_ms, 3),
                                "GBps": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1) if v["ms"] > 0 else None}
                            for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"])}}

    # end to end through the C ABI, pinned host buffers
    pin_p = torch.from_numpy(pts_h).pin_memory()
    pin_w = torch.from_numpy(w_h).pin_memory()
    pin_o = torch.empty(n, dtype=torch.int64).pin_memory()
    hp, hw, ho = pin_p.numpy(), pin_w.numpy(), pin_o.numpy().view(np.uint64)
    rcb = coupe.Rcb(iter_count=iters, tolerance=tol, mode=headline)
    for _ in range(args.warmup):
        rcb.partition(ho, (hp, hw))
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        rcb.partition(ho, (hp, hw))
    t_e2e = (time.perf_counter() - t0) / args.steps
    if world > 1:
        t = torch.tensor([t_e2e], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e = float(t.item())
    e2e_ok = bool((ho == ids_by_mode[headline]).all())

    # the partition's imbalance (coupe::imbalance) on the device: the part
    # loads of the headline ids, one pass over 16 B per point, then the
    # O(parts) rest on the host; timed per call and per kernel
    P = 1 << iters
    dids = torch.from_numpy(ids_by_mode[headline].view(np.int64)).to(dev)
    for _ in range(args.warmup):
        imb = coupe.imbalance_device(P, dids, w)
    barrier()
    ev0.record(stream)
    for _ in range(args.steps):
        imb = coupe.imbalance_device(P, dids, w)
    ev1.record(stream)
    barrier()
    t_imb = ev0.elapsed_time(ev1) / args.steps
    coupe.profile(True)
    for _ in range(args.steps):
        coupe.imbalance_device(P, dids, w)
    torch.cuda.synchronize()
    kl = coupe.profile_read().get("k_part_loads", {"ms": 0.0, "bytes": 0, "launches": 1})
    coupe.profile(False)
    k_ms = kl["ms"] / max(1, kl["launches"])
    imbalance = {"value": imb, "parts": P, "ms_per_call": round(t_imb, 4), "kernel_us": round(1e3 * k_ms, 1),
                 "kernel_GBps": round(kl["bytes"] / max(1, kl["launches"]) / (k_ms / 1e3) / 1e9, 1) if k_ms else None}

    # mesh-part's points: barycentres of a structured 160^3 hexahedral mesh
    # (4.1M elements, 262 MB of node lists), device-resident, one pass
    m = 160
    g = np.arange(m + 1, dtype=np.int64)
    idx = (g[:, None, None] * (m + 1) + g[None, :, None]) * (m + 1) + g[None, None, :]
    corners = [idx[:-1, :-1, :-1], idx[1:, :-1, :-1], idx[1:, 1:, :-1], idx[:-1, 1:, :-1],
               idx[:-1, :-1, 1:], idx[1:, :-1, 1:], idx[1:, 1:, 1:], idx[:-1, 1:, 1:]]
    d_nodes = torch.from_numpy(np.stack([c.reshape(-1) for c in corners], -1)).to(dev)
    d_coords = torch.stack(torch.meshgrid(*(torch.arange(m + 1, dtype=torch.float64, device=dev),) * 3,
                                          indexing="ij"), -1).reshape(-1, 3).contiguous()
    for _ in range(args.warmup):
        coupe.barycentres_device(d_coords, d_nodes)
    barrier()
    coupe.profile(True)
    for _ in range(args.steps):
        coupe.barycentres_device(d_coords, d_nodes)
    torch.cuda.synchronize()
    kb = coupe.profile_read().get("k_barycentres", {"ms": 0.0, "bytes": 0, "launches": 1})
    coupe.profile(False)
    b_ms = kb["ms"] / max(1, kb["launches"])
    bary = {"elements": int(d_nodes.shape[0]), "nodes_per_element": 8, "kernel_us": round(1e3 * b_ms, 1),
            "kernel_GBps": round(kb["bytes"] / max(1, kb["launches"]) / (b_ms / 1e3) / 1e9, 1) if b_ms else None}
    del d_nodes, d_coords

    # coupe's Grid::rcb: a 256^3 grid of int64 weights U{1..99} in 1024
    # parts, medians replaying 16 rayon workers
    gsz = (256, 256, 256)
    gn = 256 ** 3
    g_w = torch.from_numpy(np.random.default_rng(3).integers(1, 100, gn)).to(dev)
    g_ids = torch.zeros(gn, dtype=torch.int64, device=dev)
    for _ in range(args.warmup):
        coupe.grid_rcb_device(g_ids, g_w, gsz, 10, 16)
    barrier()
    ev0.record(stream)
    for _ in range(args.steps):
        coupe.grid_rcb_device(g_ids, g_w, gsz, 10, 16)
    ev1.record(stream)
    barrier()
    grid = {"cells": gn, "parts": 1024, "threads_replayed": 16,
            "ms_per_call": round(ev0.elapsed_time(ev1) / args.steps, 3)}
    del g_w, g_ids

    cpu = None
    parity = {}
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu, cpu_ids = cpu_baseline(pts_h, w_h, cfg)
        parity["ref32_vs_oracle_mismatches"] = int((cpu_ids != ids_by_mode["ref32"]).sum())
        import oracle  # the checker (cpu_baseline put it on the path)
        t0 = time.perf_counter()
        imb_cpu = oracle.imbalance(P, ids_by_mode[headline], w_h)
        imbalance["cpu_oracle_ms"] = round(1e3 * (time.perf_counter() - t0), 1)
        parity["imbalance_equals_oracle"] = bool(imb_cpu == imb)
    if "f32key_f64band" in ids_by_mode:
        parity["band_vs_f64_mismatches"] = int((ids_by_mode["f32key_f64band"] != ids_by_mode["f64"]).sum())
    parity["e2e_ids_equal_device_ids"] = e2e_ok

    ms = results[headline]
    value = world * n / (ms / 1e3) / 1e6
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if headline == "f32key_f64band" else "f32",
        "data": "synthetic",
        "config": _headline_config(cfg, n, pts_h.nbytes + w_h.nbytes),
        "mode": headline, "parallelism": "replicas" if world > 1 else "single",
        "modes": {m: {"ms_per_step": round(results[m], 4), "value": round(world * n / (results[m] / 1e3) / 1e6, 2)}
                  for m in results},
        "e2e": {"value": round(world * n / t_e2e / 1e6, 2), "unit": UNIT,
                "h2d_bytes_per_step": int(pts_h.nbytes + w_h.nbytes), "d2h_bytes_per_step": int(n * 8),
                "ms_per_step": round(t_e2e * 1e3, 3)},
        "gpu_launches": launches[headline],
        "roofline": roofline,
        "run": {"splits": stats["splits"], "split_steps": stats["split_steps"],
                "max_split_steps": stats["max_split_steps"], "hist_passes": stats["hist_passes"],
                "algo_bytes": stats["algo_bytes"], "kernel_launches_per_step": stats["kernel_launches"],
                "kernel_us_per_step": {m: {k: round(1e3 * v["ms"] / args.steps, 1) for k, v in pr.items()}
                                       for m, pr in by_mode.items()}},
        "parity": parity,
        "imbalance": imbalance,
        "barycentres": bary,
        "grid_rcb": grid,
        "clocks": clocks.summary() if clocks else None,
    }
    if "f32key_f64band" in results:
        line["band_vs_f64_speedup"] = round(results["f64"] / results["f32key_f64band"], 3)
    if cpu:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def _load_workload(name):
    """Host arrays and the printed description of a non-headline workload
    (both arms print the same `metric` and `config`)."""
    from coupe_gb300 import workloads
    if name == "batched4096":
        groups = workloads.batched_groups()
        n = sum(len(g[0]) for g in groups.values())
        cfg = {"workload": "batched_4096sets", "sets": 4096, "points": n, "dim": "2 and 3 (one call each)",
               "iter_count": "U{1..8} per set", "tolerance": 0.01, "weights": "int64 U{1..10}", "algorithm": "Rcb",
               "l2": _l2_note(sum(g[0].nbytes + g[1].nbytes for g in groups.values()))}
        return {"batched": True, "groups": groups, "n": n, "tol": 0.01, "cfg": cfg, "rib": False, "float": False}
    if name == "uniform1M":
        pts, w, c = workloads.uniform2d_unit()
        weights = "int64 1"
    elif name == "hexrib134M":
        pts, w, c = workloads.hex_mesh_rib()
        weights = "float64"
    else:
        pts, w, c = workloads.planes3d_lognormal()
        weights = "float64"
    rib = name == "hexrib134M"
    cfg = {"workload": c["name"], "points": len(pts), "dim": pts.shape[1], "parts": 1 << c["iter_count"],
           "iter_count": c["iter_count"], "tolerance": c["tolerance"], "weights": weights,
           "algorithm": "Rib" if rib else "Rcb", "l2": _l2_note(pts.nbytes + w.nbytes)}
    return {"batched": False, "pts": pts, "w": w, "n": len(pts), "iters": c["iter_count"], "tol": c["tolerance"],
            "cfg": cfg, "rib": rib, "float": w.dtype == np.float64}


def _l2_note(in_bytes):
    return ("L2 flushed between steps (256 MB write, untimed)" if in_bytes < L2_FLUSH_BELOW
            else "inputs larger than L2 (%d MB per step), no flush" % (in_bytes >> 20))


def _workload_metric(cfg):
    return "%s Mpoints/s, %s: FP32-key+FP64-band vs plain FP64 on GB300" % (cfg["algorithm"].upper(),
                                                                           cfg["workload"])


def run_reference_workload(args):
    """The reference arm of a non-headline workload: the oracle (OpenMP
    restatement of coupe's Rcb/Rib, f64 weights summed in f64 in rayon-like
    chunks as coupe does) on all host cores, each step a bounded sample."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    W = _load_workload(args.workload)
    cfg, n = W["cfg"], W["n"]
    kw = dict(threads=0)
    if W["float"]:
        kw["fsum"] = oracle.FSUM_SEQ
    if W["batched"]:
        groups = W["groups"]

        def run(frac):
            pts = 0
            for d, (p, w, off, it, _) in groups.items():
                k = max(1, int(round(len(it) * frac)))
                m = int(off[k])
                oracle.rcb_sets(p[:m], w[:m], off[:k + 1], it[:k], W["tol"], **kw)
                pts += m
            return pts
        unit_desc = "the first sets of each dimension's batch"
    else:
        f = oracle.rib if W["rib"] else oracle.rcb

        def run(frac):
            m = max(1 << 16, int(n * frac)) if frac < 1.0 else n
            f(W["pts"][:m], W["w"][:m], W["iters"], W["tol"], **kw)
            return m
        unit_desc = "the first points of the seeded workload"
    t0 = time.perf_counter()
    run(1.0 / 16)
    t_probe = (time.perf_counter() - t0) * 16
    frac = min(1.0, 150.0 / max(1e-9, t_probe * (args.steps + args.warmup)))
    for _ in range(max(0, args.warmup - 1)):
        run(frac)
    times, done = [], 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        done = run(frac)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    value = done / (ms / 1e3) / 1e6
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": _workload_metric(cfg), "value": round(value, 3), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if W["float"] else "f32",
        "data": "synthetic", "config": cfg,
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d of %d points per step (%s); OpenMP restatement of coupe %s on all host "
                                   "cores%s" % (done, n, unit_desc, cfg["algorithm"],
                                                "; f64 weights summed in f64 in rayon-like chunks"
                                                if W["float"] else "")},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_workload(args):
    """One line for a non-headline workload: every precision mode timed on
    device-resident inputs, the band form end to end from pinned host
    buffers, the top kernel's roofline and the oracle on the host cores."""
    import torch
    import coupe_gb300 as coupe
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    coupe.lib()
    t_gen = time.perf_counter()
    W = _load_workload(args.workload)
    cfg, n, tol = W["cfg"], W["n"], W["tol"]
    if W["batched"]:
        groups = W["groups"]
        sets = {d: (torch.from_numpy(p).to(dev), torch.from_numpy(w).to(dev), off, it)
                for d, (p, w, off, it, _) in groups.items()}
        hosts = {d: (p, w) for d, (p, w, _, _, _) in groups.items()}
        outs = {d: torch.empty(len(hosts[d][0]), dtype=torch.int64, device=dev) for d in sets}

        def step(mode):
            for d, (p, w, off, it) in sets.items():
                coupe.rcb_batched_device(outs[d], p, w, off, it, tol, mode=mode)

        def ids():
            return {d: o.cpu().numpy().view(np.uint64).copy() for d, o in outs.items()}

        def cpu_run():
            return {d: oracle.rcb_sets(p, w, off, it, tol, threads=0) for d, (p, w, off, it, _) in groups.items()}
    else:
        rib = W["rib"]
        pts_h, w_h, iters = W["pts"], W["w"], W["iters"]
        dim = pts_h.shape[1]
        hosts = {dim: (pts_h, w_h)}
        p_d, w_d = torch.from_numpy(pts_h).to(dev), torch.from_numpy(w_h).to(dev)
        out = torch.empty(n, dtype=torch.int64, device=dev)
        outs = {dim: out}

        def step(mode):
            (coupe.rib_device if rib else coupe.rcb_device)(out, p_d, w_d, iters, tol, mode=mode)

        def ids():
            return {dim: out.cpu().numpy().view(np.uint64).copy()}

        def cpu_run():
            # the reference's arithmetic: f64 weights summed in f64, in
            # chunks as rayon's fold and reduce do (threads=0: all cores);
            # Rib given the GPU's basis change, so that the comparison of
            # the ids isolates the weight sums
            kw = dict(fsum=oracle.FSUM_SEQ, threads=0, splits=True)
            if rib:
                kw["matrix"] = coupe.rib_matrix_device(p_d)
            r, st = (oracle.rib if rib else oracle.rcb)(pts_h, w_h, iters, tol, **kw)
            cpu_stats.update(st)
            cpu_stats["matrix"] = kw.get("matrix")
            return {dim: r}
    t_gen = time.perf_counter() - t_gen
    cpu_stats = {}
    tuned = None
    if W["batched"]:
        # the schedule for this batch, picked by the library's autotuner
        # (outside the timed region; ids do not depend on it)
        p, w, off, it = sets[3]
        tuned = coupe.autotune_device(outs[3], p, w, off, it, tol, mode="f32key_f64band", repeats=1)
    stream = torch.cuda.current_stream()
    in_bytes = sum(p.nbytes + w.nbytes for p, w in hosts.values())
    # inputs smaller than L2 (129 MB): every timed step starts after a
    # 256 MB write, outside its own pair of events
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev) if in_bytes < L2_FLUSH_BELOW else None
    modes = ["ref32", "f64", "f32key_f64band"]
    results, launches, got, mstats = {}, {}, {}, {}
    clocks = None
    for mode in modes:
        for _ in range(args.warmup):
            step(mode)
        torch.cuda.synchronize()
        st = coupe.last_stats()
        mstats[mode] = {k: st[k] for k in ("hist_passes", "hist_points", "band_points", "kernel_launches", "splits",
                                           "split_steps", "max_split_steps", "algo_bytes")}
        if mode == "f32key_f64band":
            clocks = Clocks(0).__enter__()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps if flush is not None else 1)]
        nl = 0
        evs[0][0].record(stream)
        for k in range(args.steps):
            if flush is not None:
                flush.fill_(k & 255)
                evs[k][0].record(stream)
            step(mode)
            nl += coupe.last_stats()["kernel_launches"]
            if flush is not None:
                evs[k][1].record(stream)
        if flush is None:
            evs[0][1].record(stream)
        torch.cuda.synchronize()
        if mode == "f32key_f64band":
            clocks.__exit__()
        results[mode] = sum(a.elapsed_time(b) for a, b in evs) / args.steps
        launches[mode] = nl
        got[mode] = ids()
    by_mode = {}
    for mode in modes:
        coupe.profile(True)
        for _ in range(args.steps):
            step(mode)
        torch.cuda.synchronize()
        by_mode[mode] = coupe.profile_read()
        coupe.profile(False)
    prof = by_mode["f32key_f64band"]
    total_ms = sum(v["ms"] for v in prof.values()) or 1.0
    top = max(prof.items(), key=lambda kv: kv[1]["ms"])
    peak, peak_kind = measured_peak()
    achieved = top[1]["bytes"] / (top[1]["ms"] / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": top[0], "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "traffic": _traffic_per_launch(top[0], "f32key_f64band", args.workload),
                "algorithmic_bytes_per_launch": top[1]["bytes"] // max(1, top[1]["launches"]),
                "launches": top[1]["launches"], "share": round(top[1]["ms"] / total_ms, 3),
                "kernels": {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                                "share": round(v["ms"] / total_ms, 3)}
                            for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"])}}
    # end to end: pinned host inputs copied in, ids copied out, every step
    pins = {d: (torch.from_numpy(p).pin_memory(), torch.from_numpy(w).pin_memory(),
                torch.empty(len(p), dtype=torch.int64).pin_memory()) for d, (p, w) in hosts.items()}
    dsts = {d: (torch.empty(tuple(p.shape), dtype=p.dtype, device=dev), torch.empty(len(w), dtype=w.dtype, device=dev))
            for d, (p, w, _) in pins.items()}

    def e2e_step():
        for d, (hp, hw, ho) in pins.items():
            dsts[d][0].copy_(hp, non_blocking=True)
            dsts[d][1].copy_(hw, non_blocking=True)
        if W["batched"]:
            for d, (_, _, off, it) in sets.items():
                coupe.rcb_batched_device(outs[d], dsts[d][0], dsts[d][1], off, it, tol, mode="f32key_f64band")
        else:
            d = next(iter(dsts))
            (coupe.rib_device if W["rib"] else coupe.rcb_device)(
                outs[d], dsts[d][0], dsts[d][1], W["iters"], tol, mode="f32key_f64band")
        for d, (_, _, ho) in pins.items():
            ho.copy_(outs[d], non_blocking=True)
        torch.cuda.synchronize()
    for _ in range(args.warmup):
        e2e_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    t_e2e = (time.perf_counter() - t0) / args.steps
    e2e_ok = all(np.array_equal(pins[d][2].numpy().view(np.uint64), got["f32key_f64band"][d]) for d in pins)
    parity = {"band_vs_f64_mismatches": int(sum((got["f32key_f64band"][d] != got["f64"][d]).sum() for d in got["f64"])),
              "e2e_ids_equal_device_ids": e2e_ok}
    cpu = None
    if not args.no_cpu:
        t0 = time.perf_counter()
        ref = cpu_run()
        t_cpu = time.perf_counter() - t0
        runs = [t_cpu]
        while sum(runs) < 2.0 and len(runs) < 50:  # short runs: the median of repeats
            t0 = time.perf_counter()
            cpu_run()
            runs.append(time.perf_counter() - t0)
        t_cpu = statistics.median(runs)
        parity["ref32_vs_oracle_mismatches"] = int(sum((ref[d] != got["ref32"][d]).sum() for d in ref))
        sample = "full workload, %s (%.3f s); OpenMP restatement of coupe %s" % (
            "one run" if len(runs) == 1 else "median of %d runs" % len(runs), t_cpu, cfg.get("algorithm", "Rcb"))
        if W["rib"]:
            sample += "; given the GPU's basis change"
        if W["float"]:
            import float_parity
            sample += "; f64 weights summed in f64 in rayon-like chunks (the reference's arithmetic)"
            # float-weight criteria of the GPU (REF32) against the reference's f64 sums
            d = next(iter(hosts))
            M = cpu_stats.get("matrix")
            keys = (oracle.map_points(hosts[d][0], M) if M is not None else hosts[d][0]).astype(np.float32)
            crit = float_parity.compare(got["ref32"][d], ref[d], keys, hosts[d][1], W["iters"], tol,
                                        cpu_stats["split_pos"])
            crit.pop("mismatch_nodes", None)
            parity["vs_reference_f64_sums"] = crit
        cpu = {"value": round(n / t_cpu / 1e6, 2), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": sample}
    ms = results["f32key_f64band"]
    h2d = sum(p.nbytes + w.nbytes for p, w in hosts.values())
    wsum = None
    if W["float"]:
        # the run's total weight against an FP64 oracle: the exact sum (the
        # oracle's 128-bit fixed point, rounded once) and the reference's
        # chunked f64 sum
        step("f32key_f64band")
        torch.cuda.synchronize()
        st = coupe.last_stats()
        w_h = hosts[next(iter(hosts))][1]
        exact = oracle.fixed_sum(w_h, oracle.fixed_scale(w_h))
        wsum = {"gpu": st["root_weight_sum"], "exact": exact, "gpu_error": st["root_weight_sum"] - exact,
                "gpu_error_bound": st["weight_sum_error_bound"]}
        if "root_sum" in cpu_stats:
            wsum["reference_f64"] = cpu_stats["root_sum"]
            wsum["reference_f64_error"] = cpu_stats["root_sum"] - exact
    line = {
        "metric": _workload_metric(cfg),
        "value": round(n / (ms / 1e3) / 1e6, 2), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic", "config": cfg,
        "modes": {m: {"ms_per_step": round(results[m], 4), "value": round(n / (results[m] / 1e3) / 1e6, 2)}
                  for m in results},
        "band_vs_f64_speedup": round(results["f64"] / results["f32key_f64band"], 3),
        "e2e": {"value": round(n / t_e2e / 1e6, 2), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(n * 8), "ms_per_step": round(t_e2e * 1e3, 3)},
        "gpu_launches": launches["f32key_f64band"], "roofline": roofline, "parity": parity,
        "run": {"last_call_stats": mstats,
                "kernel_ms_per_step": {m: {k: round(v["ms"] / args.steps, 3) for k, v in pr.items()}
                                       for m, pr in by_mode.items()}},
        "clocks": clocks.summary() if clocks else None, "generation_s": round(t_gen, 1), "autotune": tuned,
    }
    if wsum:
        line["weight_sum"] = wsum
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    return 0


def _mode_available(coupe, pts, w, part):
    try:
        coupe.rcb_device(part[:1024], pts[:1024], w[:1024], 2, 0.05, mode="f32key_f64band")
        return True
    except coupe.CoupeError:
        return False


def _traffic_per_launch(kernel, mode, workload="gauss16M"):
    """DRAM bytes per launch of `kernel` in `mode` on `workload` from the
    committed ncu summaries (profiles/traffic.json)."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            t = json.load(f)
        return t.get("%s:%s:%s" % (workload, mode, kernel))
    except Exception:
        return None


if __name__ == "__main__":
    sys.exit(main())
