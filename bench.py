#!/usr/bin/env python3
"""Benchmark of the full BVH build (bounds -> Morton -> sort -> H-PLOC -> BVH8).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload clustered12m|sphere4m|soup65k|clustered4m|batch1024]
                    [--key-bits 30|63]
                    [--radius 4|8|16]

One step = one complete build of the workload.  The default workload is the
plain clustered mesh: 12,582,912 triangles from 256 anisotropic Gaussians,
63-bit Morton codes, H-PLOC radius 8 (the configuration the >=1.5x target is
quoted on).  Inputs (453 MB) are larger than L2 (126 MB), so no flush is
needed between steps.

ours:      ``value`` = Mtris/s of nxb_build_async with the triangles resident
           in HBM, timed with CUDA events on the launching stream over K
           steps (per-stage events recorded on the same stream);
           ``e2e`` = the same metric through the reference-shaped C-ABI call
           nxb_build_bvh8 with the triangles in pinned host memory: each step
           copies them to the device, builds (allocating outputs), reads the
           result back and frees the BVH.
reference: the CPU restatement of the reference's algorithm (the oracle
           port) on all host cores: the reference has no CPU path, and its
           own CUDA build is not run on the GPU (it faulted; see
           run_reference).
Multi-GPU: the build of one mesh does not shard; each rank builds its own
replica (no collective) and ``value`` = total triangles / max rank time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

WORKLOADS = {
    "clustered12m": ("clustered12m: 12,582,912 triangles, 256 anisotropic Gaussians, lognormal(-6,1) edges", 63),
    "sphere4m": ("sphere4m: 4,194,304 triangles, 2048x1024 displaced UV sphere", 63),
    "soup65k": ("soup65k: 65,536 triangles, uniform centroids, +-0.005 vertex offsets", 30),
    "clustered4m": ("clustered4m: 4,194,304 triangles, the clustered12m generator at a third of the size "
                    "(profiling case)", 63),
    "batch1024": ("batch1024: 1024 meshes, n log-U[256, 262144] (36,469,370 triangles), each a uniform soup in "
                  "its own box (origin U[-100,100]^3, extent log-U[0.1,10])", 30),
}
BATCH_WORKLOADS = {"batch1024": (1024, 3)}
WORKLOADS["served"] = ("served: Poisson(200/s) requests, n log-U[1024, 4194304] from the soup / sphere / clustered "
                       "generators with equal probability, every 100th a 28,311,552-triangle clustered build, "
                       "32 GiB server budget", 30)

# Algorithmic bytes per triangle of each stage (k = key bytes, P = passes):
# bounds R36+W32; Morton R24 + W k + W4; sort 2P(k+4)+k; H-PLOC k+72;
# BVH8 84 + 80 * (BVH8 nodes / n).
STAGES = ["scene_bounds", "morton", "radix_sort", "hploc", "bvh8"]


def algorithmic_bytes(stage: str, k: int, passes: int, bvh8_nodes_per_tri: float) -> float:
    return {
        "scene_bounds": 68.0,
        "morton": 28.0 + k,
        "radix_sort": 2.0 * passes * (k + 4) + k,
        "hploc": k + 72.0,
        "bvh8": 84.0 + 80.0 * bvh8_nodes_per_tri,
    }[stage]


def _num(x: float, digits: int = 2):
    """Rounded float for the JSON line; None for a value that was not measured."""
    return None if x != x else round(x, digits)


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (getattr(self, "out", "") or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        loaded = [s for s in sm if s > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def make_prims(name: str) -> np.ndarray:
    from nexusbvh_gb300 import scenes
    return scenes.by_name(name)


def cpu_baseline(prims: np.ndarray, key_bits: int, radius: int, sample: int, seconds: float = 10.0) -> dict:
    """The CPU oracle (multithreaded restatement) on the whole workload (or
    its first `sample` triangles when sample > 0), built repeatedly for at
    least `seconds` of CPU work."""
    import oracle
    oracle.set_level_collapse(True)  # every stage on all host threads
    m = min(sample, prims.shape[0]) if sample > 0 else prims.shape[0]
    sub = np.ascontiguousarray(prims[:m])
    builds, stage = 0, np.zeros(5)
    t = time.perf_counter()
    while builds == 0 or time.perf_counter() - t < seconds:
        r = oracle.build(sub, key_bits, radius)
        assert r["err"] == 0
        stage += np.array(r["stage_ms"])
        builds += 1
    dt = time.perf_counter() - t
    what = "all" if m == prims.shape[0] else "the first"
    return {"value": round(m * builds / dt / 1e6, 3), "unit": "Mtris/s", "cores": oracle.threads(), "kind": "port",
            "sample": f"{what} {m:,} triangles of the workload, {builds} full CPU builds (bounds, Morton, radix sort, "
                      f"H-PLOC, BVH8) in {dt:.1f} s",
            "stage_ms": [round(x / builds, 1) for x in stage]}


def run_ours(args, world, rank, local):
    import torch

    import nexusbvh_gb300 as nxb

    torch.cuda.set_device(local)
    lib = nxb.load()
    prims_np = make_prims(args.workload)
    n = prims_np.shape[0]
    key_bits = args.key_bits
    kb = 4 if key_bits == 30 else 8
    passes = 4 if key_bits == 30 else 8
    cfg = nxb.BuildConfig(prioritize_speed=key_bits == 30, search_radius=args.radius)
    c = cfg.to_c()
    d_prims = torch.from_numpy(prims_np).cuda()
    b = nxb.Builder()
    sz = b.sizes(n, cfg)
    ws = b.workspace(sz.workspace_bytes)
    b2 = torch.empty((sz.bvh2_node_count, 32), dtype=torch.uint8, device="cuda")
    b8 = torch.empty((sz.bvh8_node_capacity, 80), dtype=torch.uint8, device="cuda")
    prim_idx = torch.empty(n, dtype=torch.int32, device="cuda")
    res = torch.zeros(64, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    sptr = int(stream.cuda_stream)

    def enqueue(events=None):
        args_ = (d_prims.data_ptr(), nxb.NXB_PRIM_TRIANGLE, n, ctypes.byref(c), ws.data_ptr(), ws.numel(),
                 b2.data_ptr(), b8.data_ptr(), prim_idx.data_ptr(), res.data_ptr(), sptr)
        if events is None:
            nxb.check(lib.nxb_build_async(*args_), "nxb_build_async")
        else:
            nxb.check(lib.nxb_build_async_timed(*args_, events), "nxb_build_async_timed")

    for _ in range(args.warmup):
        enqueue()
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(6)] for _ in range(args.steps)]
    for row in evs:  # torch creates the CUDA event on first record
        for e in row:
            e.record(stream)
    torch.cuda.synchronize()
    ev_arrays = [(ctypes.c_void_p * 6)(*[e.cuda_event for e in row]) for row in evs]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        start.record(stream)
        for k in range(args.steps):
            enqueue(ev_arrays[k])
        stop.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    elapsed = start.elapsed_time(stop)
    if world > 1:
        t = torch.tensor([elapsed], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed = float(t.item())
    result = nxb.CResult.from_buffer_copy(res.cpu().numpy().tobytes())
    if result.error_word:
        raise RuntimeError(f"device error word {result.error_word:#x}")
    stage_ms = {s: statistics.mean(evs[k][i].elapsed_time(evs[k][i + 1]) for k in range(args.steps))
                for i, s in enumerate(STAGES)}
    ms_per_step = elapsed / args.steps
    value = world * n * args.steps / elapsed / 1e3  # Mtris/s

    # e2e: host data, reference-shaped C-ABI call, result read back
    h_prims = torch.from_numpy(prims_np).pin_memory()
    d_in = torch.empty_like(d_prims)
    out = nxb.CBVH8()
    for _ in range(2):
        d_in.copy_(h_prims, non_blocking=True)
        nxb.check(lib.nxb_build_bvh8(d_in.data_ptr(), nxb.NXB_PRIM_TRIANGLE, n, ctypes.byref(c), sptr,
                                     ctypes.byref(out), None), "nxb_build_bvh8")
        nxb.check(lib.nxb_free_device_bvh8(ctypes.byref(out)), "nxb_free_device_bvh8")
    e2e_steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    copy_evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                for _ in range(e2e_steps)]
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        copy_evs[k][0].record()
        d_in.copy_(h_prims, non_blocking=True)
        copy_evs[k][1].record()
        nxb.check(lib.nxb_build_bvh8(d_in.data_ptr(), nxb.NXB_PRIM_TRIANGLE, n, ctypes.byref(c), sptr,
                                     ctypes.byref(out), None), "nxb_build_bvh8")
        nxb.check(lib.nxb_free_device_bvh8(ctypes.byref(out)), "nxb_free_device_bvh8")
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    # the host link as the e2e steps saw it (their input copies, timed on the stream)
    copy_ms = statistics.median(e0.elapsed_time(e1) for e0, e1 in copy_evs)
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * n * e2e_steps / e2e_s / 1e6

    # the same calls with the copy of step k+1 (on its own stream, into the
    # other of two input buffers) overlapping the build of step k
    copy_stream = torch.cuda.Stream()
    d_ins = [d_in, torch.empty_like(d_prims)]
    copied = [torch.cuda.Event(), torch.cuda.Event()]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with torch.cuda.stream(copy_stream):
        d_ins[0].copy_(h_prims, non_blocking=True)
    copied[0].record(copy_stream)
    for k in range(e2e_steps):
        cur = k % 2
        stream.wait_event(copied[cur])
        if k + 1 < e2e_steps:  # the other buffer's build (step k-1) has returned: the call synchronises
            with torch.cuda.stream(copy_stream):
                d_ins[1 - cur].copy_(h_prims, non_blocking=True)
            copied[1 - cur].record(copy_stream)
        nxb.check(lib.nxb_build_bvh8(d_ins[cur].data_ptr(), nxb.NXB_PRIM_TRIANGLE, n, ctypes.byref(c), sptr,
                                     ctypes.byref(out), None), "nxb_build_bvh8")
        nxb.check(lib.nxb_free_device_bvh8(ctypes.byref(out)), "nxb_free_device_bvh8")
    torch.cuda.synchronize()
    e2e_ov_s = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_ov_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ov_s = float(t.item())
    e2e_ov_value = world * n * e2e_steps / e2e_ov_s / 1e6

    # the batched and served forms, measured on the same GPU after the plain
    # line (one GPU only: with several ranks each runs the plain replica)
    forms = {}
    if world == 1 and not args.no_forms:
        del d_in, d_ins
        torch.cuda.empty_cache()
        forms["batched"] = batch_summary(measure_batch(args, 1, 0, local, steps=10, warmup=3, autotune=True,
                                                       fusion_sweep=False, loop_baseline=True))
        forms["served"] = served_summary(measure_served(args, 1, 0, local, requests=200, warmup=20, burst=1000))
    if rank != 0:
        return
    pk = peaks()
    n8_per_tri = result.bvh8_node_count / n
    per_stage = {}
    for s in STAGES:
        byts = algorithmic_bytes(s, kb, passes, n8_per_tri) * n
        gbs = byts / (stage_ms[s] * 1e-3) / 1e9
        per_stage[s] = {"ms": round(stage_ms[s], 4), "alg_bytes": int(byts), "gbs": round(gbs, 1),
                        "frac": round(gbs / pk["hbm_gbs"], 3)}
    dominant = max(STAGES, key=lambda s: stage_ms[s])
    traffic = None
    clk = clocks.summary()
    tp = ROOT / "profiles" / "dram_traffic.json"
    counters = json.loads(tp.read_text()) if tp.exists() else {}
    key = f"{args.workload}/{key_bits}/{dominant}"
    if key in counters:
        traffic = int(counters[key]["bytes_per_tri"] * n)
    # issue side of the latency-bound kernels: warp instructions per launch
    # (ncu count per triangle, scaled) against the SMs' issue slots
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    mhz = clk.get("sm_mhz") or 2070.0
    for stg in ("hploc", "bvh8"):
        c = counters.get(f"{args.workload}/{key_bits}/{stg}", {})
        if "warp_inst_per_tri" in c:
            inst = c["warp_inst_per_tri"] * n
            per_stage[stg]["warp_inst"] = int(inst)
            per_stage[stg]["issue_frac"] = round(inst / (stage_ms[stg] * 1e-3 * sms * 4 * mhz * 1e6), 3)
    line = {
        "metric": "Mtris/s full build (bounds, Morton, radix sort, H-PLOC BVH2, BVH8)",
        "value": round(value, 2),
        "unit": "Mtris/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded generators standing in for the reference's scene files)",
        "config": {
            "workload": WORKLOADS[args.workload][0],
            "n_tris": n,
            "key_bits": key_bits,
            "search_radius": args.radius,
            "parallelism": f"replicas x{world} (one mesh per GPU, no collective)",
            "l2": "inputs larger than L2 (triangles 36 B x n, no flush needed)",
            "stage_ms": {s: per_stage[s]["ms"] for s in STAGES},
            "stage_sum_ms": round(sum(stage_ms.values()), 4),
            "stage_roofline": per_stage,
            "bvh8_nodes": int(result.bvh8_node_count),
            "e2e_overlapped_copy": {"value": round(e2e_ov_value, 2), "unit": "Mtris/s",
                                    "how": "the e2e calls with step k+1's host->device copy on a second stream "
                                           "overlapping step k's build (supplementary; e2e is the serial loop)"},
            **forms,
        },
        "roofline": {
            "kernel": dominant,
            "bound": "hbm",
            "achieved": per_stage[dominant]["gbs"],
            "peak": pk["hbm_gbs"],
            "unit": "GB/s",
            "frac": per_stage[dominant]["frac"],
            "traffic": traffic,
            "peak_source": pk["source"],
            "issue_frac": per_stage[dominant].get("issue_frac"),
            **({"traffic_note": "includes the 64 B/tri child-pair records H-PLOC writes for the BVH8 "
                                "collapse, which then reads them instead of the BVH2 nodes"}
               if dominant == "hploc" and traffic else {}),
        },
        "e2e": {"value": round(e2e_value, 2), "unit": "Mtris/s", "h2d_bytes_per_step": 36 * n,
                "d2h_bytes_per_step": ctypes.sizeof(nxb.CResult),
                "call": "nxb_build_bvh8 (C ABI, allocates outputs) after a pinned host->device copy",
                "copy_ms": round(copy_ms, 3), "h2d_gbs": round(36 * n / (copy_ms * 1e-3) / 1e9, 1)},
        # per build: bounds, Morton, the sort (30-bit: 4 passes; 63-bit: 4
        # passes, the bucket sort and the fallback launch), H-PLOC (which
        # also initialises the BVH8 work queue), BVH8, finalize
        "gpu_launches": (5 + (4 if key_bits == 30 else 6)) * args.steps,
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(prims_np, key_bits, args.radius, args.cpu_sample)
    print(json.dumps(line), flush=True)


def measure_batch(args, world, rank, local, steps: int, warmup: int, autotune: bool, fusion_sweep: bool,
                  loop_baseline: bool, cpu_baseline_tris: int = 0) -> dict:
    """The batched form on the batch1024 meshes: all meshes in one
    graph-replayed pipeline (nxb_batch_*), next to a loop of plain builds over
    the same meshes.  Returns the measurements (rank 0's line fields)."""
    import torch
    import nexusbvh_gb300 as nxb
    from nexusbvh_gb300 import scenes

    from nexusbvh_gb300 import dist

    torch.cuda.set_device(local)
    lib = nxb.load()
    meshes_all, seed = BATCH_WORKLOADS["batch1024"]
    counts_all = scenes.batch_counts(meshes_all, seed=seed)
    prims_all = scenes.batch_meshes(counts_all, seed=seed)
    n_all = prims_all.shape[0]
    # N GPUs: each rank builds a disjoint, size-balanced share of the meshes
    # (no collective; whole-job rate = all triangles / slowest rank)
    mine = dist.shard_meshes(counts_all, world, rank) if world > 1 else np.arange(meshes_all)
    off_all = np.concatenate([[0], np.cumsum(counts_all)]).astype(np.int64)
    counts = counts_all[mine]
    prims_np = np.concatenate([prims_all[off_all[m]:off_all[m + 1]] for m in mine]) if world > 1 else prims_all
    meshes = len(mine)
    n = prims_np.shape[0]
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    d_prims = torch.from_numpy(prims_np).cuda()
    stream = torch.cuda.current_stream()
    sptr = int(stream.cuda_stream)
    batch = nxb.Batch(counts, config=nxb.BuildConfig(prioritize_speed=True, search_radius=args.radius))
    t_tune = time.perf_counter()
    tuning = batch.autotune(d_prims, repeats=2) if autotune else batch.tuning()
    t_tune = time.perf_counter() - t_tune

    def timed_build(groups: int, reps: int = 5) -> float:
        """Median ms of a build with the chosen tuning but the given fusion point."""
        t = batch.tuning()
        t.fusion_groups = groups
        batch.set_tuning(t)
        batch.build(d_prims)
        ms = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            batch.build_async(d_prims)
            e1.record()
            batch.wait(results=False)
            ms.append(e0.elapsed_time(e1))
        return statistics.median(ms)

    chosen = batch.tuning()
    fusion = {f"groups_{g}_ms": round(timed_build(g), 4) for g in (1, 2, 4, 8)} if fusion_sweep else None
    batch.set_tuning(chosen)
    for _ in range(warmup):
        batch.build_async(d_prims)
    batch.wait(results=False)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        start.record(stream)
        for _ in range(steps):
            batch.build_async(d_prims)
        stop.record(stream)
        torch.cuda.synchronize()
    res = batch.wait(results=True)
    elapsed = start.elapsed_time(stop)
    value = dist.whole_job_rate(n * steps, elapsed * 1e-3, device="cuda") / 1e6
    elapsed = dist.max_over_ranks(elapsed, device="cuda")
    n8 = sum(r.bvh8_node_count for r in res)

    # e2e: pinned host triangles -> device, batch build, per-mesh results back
    h_prims = torch.from_numpy(prims_np).pin_memory()
    d_in = torch.empty_like(d_prims)
    d_in.copy_(h_prims, non_blocking=True)
    batch.build(d_in)  # capture for this buffer
    e2e_steps = max(3, min(steps, 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        d_in.copy_(h_prims, non_blocking=True)
        batch.build(d_in)
    e2e_s = time.perf_counter() - t0
    e2e_value = dist.whole_job_rate(n * e2e_steps, e2e_s, device="cuda") / 1e6
    del d_in, h_prims

    # the loop of plain builds the batch replaces: the reference-shaped call
    # per mesh (allocating, synchronising), and nxb_build_async per mesh into
    # one resident workspace (no per-mesh synchronisation)
    cfg = nxb.BuildConfig(prioritize_speed=True, search_radius=args.radius)
    c = cfg.to_c()
    out = nxb.CBVH8()

    def loop_plain():
        for m in range(meshes):
            k = int(counts[m])
            if k == 0:
                continue
            ptr = d_prims.data_ptr() + int(off[m]) * 36
            nxb.check(lib.nxb_build_bvh8(ptr, nxb.NXB_PRIM_TRIANGLE, k, ctypes.byref(c), sptr, ctypes.byref(out),
                                         None), "nxb_build_bvh8")
            nxb.check(lib.nxb_free_device_bvh8(ctypes.byref(out)), "nxb_free_device_bvh8")

    t_loop = t_loop_async = float("nan")
    if loop_baseline:
        b = nxb.Builder()
        big = int(max(counts))
        sz = b.sizes(big, cfg)
        ws = b.workspace(sz.workspace_bytes)
        b2 = torch.empty((sz.bvh2_node_count, 32), dtype=torch.uint8, device="cuda")
        b8 = torch.empty((sz.bvh8_node_capacity, 80), dtype=torch.uint8, device="cuda")
        pidx = torch.empty(big, dtype=torch.int32, device="cuda")
        rbuf = torch.zeros(64, dtype=torch.uint8, device="cuda")

        def loop_async():
            for m in range(meshes):
                k = int(counts[m])
                if k == 0:
                    continue
                ptr = d_prims.data_ptr() + int(off[m]) * 36
                nxb.check(lib.nxb_build_async(ptr, nxb.NXB_PRIM_TRIANGLE, k, ctypes.byref(c), ws.data_ptr(),
                                              ws.numel(), b2.data_ptr(), b8.data_ptr(), pidx.data_ptr(),
                                              rbuf.data_ptr(), sptr), "nxb_build_async")

        loop_plain()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loop_plain()
        torch.cuda.synchronize()
        t_loop = time.perf_counter() - t0
        loop_async()
        torch.cuda.synchronize()
        start.record(stream)
        loop_async()
        stop.record(stream)
        torch.cuda.synchronize()
        t_loop_async = start.elapsed_time(stop) / 1e3
        del ws, b2, b8, pidx, rbuf
    passes = -(-(30 + max(1, (meshes - 1).bit_length())) // int(tuning.sort_digit_bits))
    per_tri = (algorithmic_bytes("scene_bounds", 8, passes, 0) + algorithmic_bytes("morton", 8, passes, 0)
               + 4.0 + algorithmic_bytes("radix_sort", 8, passes, 0) + algorithmic_bytes("hploc", 8, passes, 0)
               + algorithmic_bytes("bvh8", 8, passes, n8 / n))
    ms = elapsed / steps
    out_d = {
        "value": value, "ms": ms, "n": n, "n_all": n_all, "meshes": meshes, "meshes_all": meshes_all,
        "tuning": tuning, "passes": passes, "fusion": fusion, "t_tune": t_tune, "n8": n8,
        "gbs": per_tri * n / (ms * 1e-3) / 1e9, "e2e": e2e_value, "t_loop": t_loop, "t_loop_async": t_loop_async,
        "clocks": clocks.summary(),
    }
    if cpu_baseline_tris and rank == 0:
        import oracle
        oracle.set_level_collapse(True)
        t = time.perf_counter()
        done = 0
        m = 0
        while done < cpu_baseline_tris and m < meshes:
            k = int(counts[m])
            if k:
                r = oracle.build(np.ascontiguousarray(prims_np[off[m]:off[m + 1]]), 30, args.radius)
                assert r["err"] == 0
                done += k
            m += 1
        dt = time.perf_counter() - t
        out_d["cpu_baseline"] = {"value": round(done / dt / 1e6, 3), "unit": "Mtris/s", "cores": oracle.threads(),
                                 "kind": "port", "sample": f"the first {m} meshes ({done:,} triangles), one CPU "
                                                           f"build each, in {dt:.2f} s"}
    del d_prims, batch
    torch.cuda.empty_cache()
    return out_d


def batch_summary(b: dict) -> dict:
    """The batched measurements as a compact record."""
    t = b["tuning"]
    return {
        "mtris_s": round(b["value"], 2), "ms_per_build": round(b["ms"], 4), "meshes": b["meshes_all"],
        "n_tris": b["n_all"],
        "tuning": {"sort_digit_bits": int(t.sort_digit_bits), "sort_passes": b["passes"],
                   "search_radius": int(t.search_radius), "hploc_ctas_per_sm": int(t.hploc_ctas_per_sm),
                   "fusion_groups": int(t.fusion_groups), "block_size": int(t.block_size),
                   "candidates": int(t.candidates_tried), "tune_s": round(b["t_tune"], 2)},
        "loop_plain_api_ms": _num(b["t_loop"] * 1e3),
        "loop_async_ms": _num(b["t_loop_async"] * 1e3),
        "speedup_vs_loop_plain_api": _num(b["t_loop"] * 1e3 / b["ms"]),
        "speedup_vs_loop_async": _num(b["t_loop_async"] * 1e3 / b["ms"]),
        "target_speedup": 3.0,
        "e2e_mtris_s": round(b["e2e"], 2),
    }


def run_batch(args, world, rank, local):
    """Batched form: the batch1024 line."""
    b = measure_batch(args, world, rank, local, args.steps, args.warmup, autotune=not args.no_autotune,
                      fusion_sweep=not args.no_autotune, loop_baseline=not args.no_loop_baseline,
                      cpu_baseline_tris=0 if args.no_cpu_baseline else (args.cpu_sample or 1 << 62))
    if rank != 0:
        return
    pk = peaks()
    tuning, meshes, n = b["tuning"], b["meshes"], b["n"]
    line = {
        "metric": "Mtris/s batched build (1024 meshes, bounds, Morton, radix sort, H-PLOC BVH2, BVH8)",
        "value": round(b["value"], 2), "unit": "Mtris/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(b["ms"], 4), "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generators standing in for the reference's scene files)",
        "config": {
            "workload": WORKLOADS[args.workload][0], "meshes": b["meshes_all"], "n_tris": b["n_all"],
            "rank0_meshes": meshes, "rank0_tris": n, "key_bits": 30,
            "search_radius": int(tuning.search_radius),
            "parallelism": f"meshes sharded over {world} GPU(s) by size, no collective",
            "l2": "inputs larger than L2 (1.3 GB of triangles), no flush needed",
            "tuning": dict(batch_summary(b)["tuning"], fusion_point=b["fusion"]),
            "bvh8_nodes": int(b["n8"]),
            "loop_plain_api_ms": _num(b["t_loop"] * 1e3),
            "loop_plain_api_mtris_s": _num(n / b["t_loop"] / 1e6),
            "loop_async_ms": _num(b["t_loop_async"] * 1e3),
            "speedup_vs_loop_plain_api": _num(b["t_loop"] * 1e3 / b["ms"]),
            "speedup_vs_loop_async": _num(b["t_loop_async"] * 1e3 / b["ms"]),
        },
        "roofline": {"kernel": "whole batched pipeline", "bound": "hbm", "achieved": round(b["gbs"], 1),
                     "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": round(b["gbs"] / pk["hbm_gbs"], 3),
                     "traffic": None, "peak_source": pk["source"]},
        "e2e": {"value": round(b["e2e"], 2), "unit": "Mtris/s", "h2d_bytes_per_step": 36 * n,
                "d2h_bytes_per_step": 52 * meshes + 4,
                "call": "nxb_batch_build (graph replay + wait + per-mesh results) after a pinned host->device copy"},
        # per build: tile ranges, bounds, Morton, the sort passes, BVH8 queue
        # init, H-PLOC, BVH8, finalize (one mesh group)
        "gpu_launches": (7 + b["passes"]) * args.steps,
        "clocks": b["clocks"],
    }
    if "cpu_baseline" in b:
        line["cpu_baseline"] = b["cpu_baseline"]
    print(json.dumps(line), flush=True)


def served_requests(count: int, seed: int = 11):
    """(kind, n, key_bits) of each request: kind 0 soup, 1 sphere, 2 clustered,
    3 the 28,311,552-triangle clustered build every 100th request."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        if i % 100 == 99:
            out.append((3, 28_311_552, 63))
            continue
        kind = int(rng.integers(0, 3))
        n = int(np.exp(rng.uniform(np.log(1024), np.log(4_194_304 + 1))))
        key_bits = 30 if kind == 0 else (63 if kind == 2 else int(rng.choice([30, 63])))
        out.append((kind, min(n, 4_194_304), key_bits))
    return out


def burst_requests(count: int, seed: int = 21):
    """(kind, n, key_bits) of a burst of small requests: configuration-0 and
    -1 style meshes (kind 0 soup, kind 1 sphere, alternating), n log-U[1024,
    65536], 30-bit codes (the size and key width the server may batch)."""
    rng = np.random.default_rng(seed)
    return [(i % 2, int(np.exp(rng.uniform(np.log(1024), np.log(65536 + 1)))), 30) for i in range(count)]


def _pctl(x, q):
    return float(np.percentile(x, q)) if len(x) else float("nan")


def measure_served(args, world, rank, local, requests: int, warmup: int, burst: int = 1000) -> dict:
    """Served form: a build server (nxb_server_*) fed Poisson arrivals (200
    requests/s, the configuration's stream) and a burst of small requests
    that arrives faster than the GPU serves them; per request latency =
    submit -> completion.  Each pass is compared with the same arrivals
    served by serial plain builds."""
    import threading
    import queue as _q
    import torch
    import nexusbvh_gb300 as nxb
    from nexusbvh_gb300 import scenes

    torch.cuda.set_device(local)
    lib = nxb.load()
    pools = [scenes.uniform_soup(4_194_304, seed=0), scenes.displaced_sphere(2048, 1024, seed=1),
             scenes.clustered(4_194_304, seed=2), scenes.clustered(28_311_552, seed=5)]
    host = [torch.from_numpy(p).pin_memory() for p in pools]
    dev = [t.cuda() for t in host]
    del pools
    stream_ptr = int(torch.cuda.current_stream().cuda_stream)

    def arrivals_of(gaps):
        return np.cumsum(gaps)

    def serve(reqs, gaps, warm, on_device):
        srv = nxb.Server(budget_bytes=32 << 30, reserve=True)
        results = []
        tickets_q = _q.Queue()

        def drain():
            for i, t in enumerate(iter(tickets_q.get, None)):
                r = srv.wait(t)
                if i >= warm:
                    results.append((r.latency_ms, r.queue_ms, r.batched_with, r.device_start_ms,
                                    r.device_end_ms))
                srv.release(t)

        th = threading.Thread(target=drain)
        th.start()
        t0 = time.perf_counter()
        arr = t0 + arrivals_of(gaps)
        start_timed = None
        for i, (kind, n, kb) in enumerate(reqs):
            wait = arr[i] - time.perf_counter()
            if wait > 0.0005:
                time.sleep(wait - 0.0003)  # leave the GIL to the draining thread
            while time.perf_counter() < arr[i]:
                pass
            if i == warm:
                start_timed = time.perf_counter()
            cfg = nxb.BuildConfig(prioritize_speed=kb == 30)
            t = srv.submit(dev[kind][:n] if on_device else host[kind][:n].numpy(), cfg)
            tickets_q.put(t)
        tickets_q.put(None)
        th.join()
        wall = time.perf_counter() - (start_timed or t0)
        st = srv.stats()
        srv.close()
        lat = [r[0] for r in results]
        # jobs (distinct device intervals) whose GPU work overlapped another job's
        jobs = sorted({(r[3], r[4]) for r in results})
        overl = sum(1 for k, a in enumerate(jobs) if any(max(a[0], b[0]) < min(a[1], b[1])
                                                         for b in jobs[max(0, k - 64):k + 64] if b != a))
        tris = sum(n for _, n, _ in reqs[warm:])
        return {"p50_ms": _pctl(lat, 50), "p99_ms": _pctl(lat, 99), "mean_ms": float(np.mean(lat)),
                "max_ms": float(np.max(lat)), "queue_p99_ms": _pctl([r[1] for r in results], 99),
                "requests": len(lat), "batched_requests": sum(1 for r in results if r[2] > 1),
                "wall_s": wall, "builds_s": len(lat) / wall, "mtris_s": tris / wall / 1e6,
                "gpu_jobs": len(jobs), "jobs_overlapping_another": overl,
                "peak_bytes": int(st.peak_bytes_in_use), "builds": int(st.builds),
                "batched_builds": int(st.batched_builds)}

    def serial(reqs, gaps, warm, on_device):
        """The same arrivals served by serial plain builds (the reference's
        model: one nxb_build_bvh8 call at a time), inputs resident on the
        device or copied from pinned host memory before each build."""
        out = nxb.CBVH8()
        lat = []
        copies = []  # (bytes, start event, end event) of the large host-input copies
        d_in = torch.empty((max(n for _, n, _ in reqs), 9), dtype=torch.float32, device="cuda")
        t0 = time.perf_counter()
        arr = t0 + arrivals_of(gaps)
        start_timed = None
        for i, (kind, n, kb) in enumerate(reqs):
            while time.perf_counter() < arr[i]:
                pass
            if i == warm:
                start_timed = time.perf_counter()
            c = nxb.BuildConfig(prioritize_speed=kb == 30).to_c()
            src = dev[kind]
            if not on_device:
                ev = None
                if i >= warm and n >= 1_000_000:
                    ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                    ev[0].record()
                d_in[:n].copy_(host[kind][:n], non_blocking=True)
                if ev:
                    ev[1].record()
                    copies.append((36 * n, ev[0], ev[1]))
                src = d_in
            nxb.check(lib.nxb_build_bvh8(src.data_ptr(), nxb.NXB_PRIM_TRIANGLE, n, ctypes.byref(c),
                                         stream_ptr, ctypes.byref(out), None), "nxb_build_bvh8")
            nxb.check(lib.nxb_free_device_bvh8(ctypes.byref(out)), "nxb_free_device_bvh8")
            if i >= warm:
                lat.append((time.perf_counter() - arr[i]) * 1e3)
        wall = time.perf_counter() - (start_timed or t0)
        tris = sum(n for _, n, _ in reqs[warm:])
        r = {"p50_ms": _pctl(lat, 50), "p99_ms": _pctl(lat, 99), "mean_ms": float(np.mean(lat)),
             "max_ms": float(np.max(lat)), "wall_s": wall, "builds_s": len(lat) / wall,
             "mtris_s": tris / wall / 1e6}
        if copies:
            # the host link as this pass saw it: GB/s of each large input copy
            torch.cuda.synchronize()
            gbs = [b / (e0.elapsed_time(e1) * 1e-3) / 1e9 for b, e0, e1 in copies]
            r["h2d_gbs_min"] = float(np.min(gbs))
            r["h2d_gbs_median"] = float(np.median(gbs))
            r["h2d_copies"] = len(gbs)
        return r

    total = warmup + requests
    reqs = served_requests(total)
    gaps = np.random.default_rng(12).exponential(1.0 / 200.0, size=total)
    out = {}
    with ClockSampler(local) as clocks:
        out["device_resident"] = serve(reqs, gaps, warmup, True)
        out["host_input"] = serve(reqs, gaps, warmup, False)
        out["serial_plain_device"] = serial(reqs, gaps, warmup, True)
        out["serial_plain_host"] = serial(reqs, gaps, warmup, False)
        if burst:
            breqs = burst_requests(burst + 20)
            bgaps = np.random.default_rng(22).exponential(1.0 / 20_000.0, size=len(breqs))
            out["burst"] = serve(breqs, bgaps, 20, True)
            out["burst_serial_plain"] = serial(breqs, bgaps, 20, True)
    out["clocks"] = clocks.summary()
    out["reqs"] = reqs
    out["warmup"] = warmup
    del dev, host
    torch.cuda.empty_cache()
    return out


def served_summary(sv: dict) -> dict:
    def r(d):
        return {k: (round(v, 3) if isinstance(v, float) else v) for k, v in d.items()}
    keys = ["device_resident", "host_input", "serial_plain_device", "serial_plain_host", "burst",
            "burst_serial_plain"]
    return {k: r(sv[k]) for k in keys if k in sv}


def run_served(args, world, rank, local):
    """Served form: the served line (p99 latency of device-resident requests)."""
    sv = measure_served(args, world, rank, local, args.steps, args.warmup)
    if rank != 0:
        return
    reqs, warm = sv["reqs"], sv["warmup"]
    resident, hostin = sv["device_resident"], sv["host_input"]
    n_big = sum(1 for k, _, _ in reqs[warm:] if k == 3)
    line = {
        "metric": "p99 request latency, served builds (submit -> BVH8 done)",
        "value": round(resident["p99_ms"], 3), "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(resident["mean_ms"], 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generators standing in for the reference's scene files)",
        "config": dict({"workload": WORKLOADS["served"][0], "requests": args.steps, "big_requests": n_big,
                        "budget_gib": 32, "streams": 4, "batch_max_prims": 65536,
                        "l2": "each request's input is streamed once; the big builds exceed L2",
                        "burst": "1,000 requests of configuration-0/1 meshes (n log-U[1024, 65536], 30-bit) "
                                 "arriving at 20,000/s"},
                       **served_summary(sv)),
        "roofline": None,
        "e2e": {"value": round(hostin["p99_ms"], 3), "unit": "ms",
                "h2d_bytes_per_step": int(np.mean([n * 36 for _, n, _ in reqs[warm:]])),
                "d2h_bytes_per_step": 40,
                "call": "nxb_server_submit with host (pinned) input, nxb_server_wait, nxb_server_release"},
        "gpu_launches": None,
        "clocks": sv["clocks"],
    }
    print(json.dumps(line), flush=True)


def run_reference(args, world, rank, local):
    """The reference arm.  The reference's path has no CPU implementation,
    and its own CUDA build is not run on the GPU any more: its H-PLOC kernel
    reads cluster ids and node boxes written by other SMs with plain
    L1-cacheable loads (NexusBVH/src/Cuda/BinaryBuilder.cu:51,185), and it
    faulted (Xid 31) on the 4,194,304-triangle sphere with 30-bit keys.
    What is timed here is therefore the CPU restatement of the reference's
    algorithm (the oracle port) on all host cores, each step one CPU build
    of the whole workload (a prefix of it only when the steps would not
    fit the time budget)."""
    if rank != 0:
        return
    if args.workload == "served":
        print(json.dumps({"impl": "reference", "unavailable": "the served form (a build server with admission and "
                          "continuous batching) has no counterpart in the reference, which is a per-mesh library "
                          "call"}), flush=True)
        return
    import oracle
    oracle.set_level_collapse(True)  # every stage on all host threads

    key_bits = args.key_bits
    if args.workload in BATCH_WORKLOADS:
        from nexusbvh_gb300 import scenes
        meshes, seed = BATCH_WORKLOADS[args.workload]
        counts = scenes.batch_counts(meshes, seed=seed)
        prims_np = scenes.batch_meshes(counts, seed=seed)
        off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    else:
        prims_np = make_prims(args.workload)
        counts = np.array([prims_np.shape[0]])
        off = np.array([0, prims_np.shape[0]], dtype=np.int64)
    n = prims_np.shape[0]

    def sample_of(tris: int):
        """The step's sample: the first `tris` triangles, each mesh built on
        its own (a batch's meshes whole, one mesh cut at a prefix)."""
        if len(counts) == 1:
            return [np.ascontiguousarray(prims_np[:max(1, min(tris, n))])]
        last = max(1, min(int(np.searchsorted(off, min(tris, off[-1]), side="left")), len(counts)))
        return [np.ascontiguousarray(prims_np[off[i]:off[i + 1]]) for i in range(last) if counts[i]]

    def step(subs):
        st = np.zeros(5)
        for x in subs:
            r = oracle.build(x, key_bits, args.radius)
            assert r["err"] == 0
            st += np.array(r["stage_ms"])
        return st

    for _ in range(args.warmup):
        oracle.build(prims_np[: min(n, 65536)], key_bits, args.radius)
    # Each step builds the whole workload when steps x (one whole build)
    # fits the time budget, else the largest prefix that does: one whole
    # build, untimed, measures it.
    subs = sample_of(args.cpu_sample or n)
    if not args.cpu_sample:
        t = time.perf_counter()
        step(subs)
        t_full = time.perf_counter() - t
        if args.steps * t_full > args.cpu_budget:
            subs = sample_of(int(n * args.cpu_budget / (args.steps * t_full)))
    m = sum(x.shape[0] for x in subs)
    times = []
    stage = np.zeros(5)
    for _ in range(args.steps):
        t = time.perf_counter()
        stage += step(subs)
        times.append(time.perf_counter() - t)
    total = sum(times)
    value = m * args.steps / total / 1e6
    line = {"metric": "Mtris/s full build (bounds, Morton, radix sort, H-PLOC BVH2, BVH8)", "value": round(value, 3),
            "unit": "Mtris/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(total / args.steps * 1e3, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "impl": "reference",
            "data": "synthetic (seeded generators standing in for the reference's scene files)",
            "config": {"workload": WORKLOADS[args.workload][0], "n_tris": n, "key_bits": key_bits,
                       "search_radius": args.radius, "sample_tris": m},
            "cpu_baseline": {"value": round(value, 3), "unit": "Mtris/s", "cores": oracle.threads(), "kind": "port",
                             "sample": (f"all {n:,} triangles of the workload" if m == n else
                                        f"first {m:,} of the workload's {n:,} triangles") +
                                       " per step, one full CPU build (bounds, Morton, radix sort, H-PLOC, BVH8)"
                                       + (" of each mesh" if len(counts) > 1 else ""),
                             "stage_ms": [round(x / args.steps, 1) for x in stage]},
            "e2e": {"value": round(value, 3), "unit": "Mtris/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference path has no CPU implementation; its CUDA build faulted on GB300 (Xid 31, stale-L1 "
                    "race in BinaryBuilder.cu) and is not run again; the CPU port of its algorithm is timed"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="clustered12m")
    ap.add_argument("--key-bits", type=int, choices=[30, 63], default=None)
    ap.add_argument("--radius", type=int, choices=[4, 8, 16], default=8)
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="CPU builds: triangles per sample (0: the whole workload; the reference arm then shrinks it "
                         "to a prefix only if --steps whole builds would exceed --cpu-budget)")
    ap.add_argument("--cpu-budget", type=float, default=150.0,
                    help="reference arm: seconds of timed CPU steps to aim below")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-loop-baseline", action="store_true",
                    help="batched workloads: leave out the loop-of-plain-builds comparison")
    ap.add_argument("--no-autotune", action="store_true",
                    help="batched workloads: build with the default tuning instead of tuning first")
    ap.add_argument("--no-forms", action="store_true",
                    help="plain workloads: leave out the batched and served records of the line")
    args = ap.parse_args()
    if args.key_bits is None:
        args.key_bits = WORKLOADS[args.workload][1]
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist()
    if world > 1:
        import torch
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    try:
        if args.impl == "reference":
            run_reference(args, world, rank, local)
        elif args.workload in BATCH_WORKLOADS:
            run_batch(args, world, rank, local)
        elif args.workload == "served":
            run_served(args, world, rank, local)
        else:
            run_ours(args, world, rank, local)
    finally:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
