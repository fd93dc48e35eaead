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
    """The CPU oracle (multithreaded restatement) on a bounded prefix sample,
    built repeatedly for at least `seconds` of CPU work."""
    import oracle
    oracle.set_level_collapse(True)  # every stage on all host threads
    m = min(sample, prims.shape[0])
    sub = np.ascontiguousarray(prims[:m])
    builds, stage = 0, np.zeros(5)
    t = time.perf_counter()
    while builds == 0 or time.perf_counter() - t < seconds:
        r = oracle.build(sub, key_bits, radius)
        assert r["err"] == 0
        stage += np.array(r["stage_ms"])
        builds += 1
    dt = time.perf_counter() - t
    return {"value": round(m * builds / dt / 1e6, 3), "unit": "Mtris/s", "cores": oracle.threads(), "kind": "port",
            "sample": f"first {m:,} triangles of the workload, {builds} full CPU builds (bounds, Morton, radix sort, "
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
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        d_in.copy_(h_prims, non_blocking=True)
        nxb.check(lib.nxb_build_bvh8(d_in.data_ptr(), nxb.NXB_PRIM_TRIANGLE, n, ctypes.byref(c), sptr,
                                     ctypes.byref(out), None), "nxb_build_bvh8")
        nxb.check(lib.nxb_free_device_bvh8(ctypes.byref(out)), "nxb_free_device_bvh8")
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
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
    tp = ROOT / "profiles" / "dram_traffic.json"
    if tp.exists():
        tj = json.loads(tp.read_text())
        key = f"{args.workload}/{key_bits}/{dominant}"
        if key in tj:
            traffic = int(tj[key]["bytes_per_tri"] * n)
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
        },
        "e2e": {"value": round(e2e_value, 2), "unit": "Mtris/s", "h2d_bytes_per_step": 36 * n,
                "d2h_bytes_per_step": ctypes.sizeof(nxb.CResult),
                "call": "nxb_build_bvh8 (C ABI, allocates outputs) after a pinned host->device copy"},
        "gpu_launches": (6 + passes) * args.steps,
        "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(prims_np, key_bits, args.radius, args.cpu_sample)
    print(json.dumps(line), flush=True)


def run_batch(args, world, rank, local):
    """Batched form: all meshes in one graph-replayed pipeline (nxb_batch_*),
    next to a loop of plain builds over the same meshes."""
    import torch
    import nexusbvh_gb300 as nxb
    from nexusbvh_gb300 import scenes

    from nexusbvh_gb300 import dist

    torch.cuda.set_device(local)
    lib = nxb.load()
    meshes_all, seed = BATCH_WORKLOADS[args.workload]
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
    tuning = batch.tuning() if args.no_autotune else batch.autotune(d_prims, repeats=2)
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
    # the fusion-point sweep is part of the tuning report (skipped with --no-autotune)
    fusion = None if args.no_autotune else {f"groups_{g}_ms": round(timed_build(g), 4) for g in (1, 2, 4, 8)}
    batch.set_tuning(chosen)
    for _ in range(args.warmup):
        batch.build_async(d_prims)
    batch.wait(results=False)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        start.record(stream)
        for _ in range(args.steps):
            batch.build_async(d_prims)
        stop.record(stream)
        torch.cuda.synchronize()
    res = batch.wait(results=True)
    elapsed = start.elapsed_time(stop)
    value = dist.whole_job_rate(n * args.steps, elapsed * 1e-3, device="cuda") / 1e6
    elapsed = dist.max_over_ranks(elapsed, device="cuda")
    n8 = sum(r.bvh8_node_count for r in res)

    # e2e: pinned host triangles -> device, batch build, per-mesh results back
    h_prims = torch.from_numpy(prims_np).pin_memory()
    d_in = torch.empty_like(d_prims)
    d_in.copy_(h_prims, non_blocking=True)
    batch.build(d_in)  # capture for this buffer
    e2e_steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        d_in.copy_(h_prims, non_blocking=True)
        batch.build(d_in)
    e2e_s = time.perf_counter() - t0
    e2e_value = dist.whole_job_rate(n * e2e_steps, e2e_s, device="cuda") / 1e6

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
            nxb.check(lib.nxb_build_async(ptr, nxb.NXB_PRIM_TRIANGLE, k, ctypes.byref(c), ws.data_ptr(), ws.numel(),
                                          b2.data_ptr(), b8.data_ptr(), pidx.data_ptr(), rbuf.data_ptr(), sptr),
                      "nxb_build_async")

    t_loop = t_loop_async = float("nan")
    if not args.no_loop_baseline:
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
    if rank != 0:
        return
    pk = peaks()
    passes = -(-(30 + max(1, (meshes - 1).bit_length())) // int(tuning.sort_digit_bits))
    per_tri = (algorithmic_bytes("scene_bounds", 8, passes, 0) + algorithmic_bytes("morton", 8, passes, 0)
               + 4.0 + algorithmic_bytes("radix_sort", 8, passes, 0) + algorithmic_bytes("hploc", 8, passes, 0)
               + algorithmic_bytes("bvh8", 8, passes, n8 / n))
    ms = elapsed / args.steps
    gbs = per_tri * n / (ms * 1e-3) / 1e9
    line = {
        "metric": "Mtris/s batched build (1024 meshes, bounds, Morton, radix sort, H-PLOC BVH2, BVH8)",
        "value": round(value, 2), "unit": "Mtris/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded generators standing in for the reference's scene files)",
        "config": {
            "workload": WORKLOADS[args.workload][0], "meshes": meshes_all, "n_tris": n_all,
            "rank0_meshes": meshes, "rank0_tris": n, "key_bits": 30,
            "search_radius": int(tuning.search_radius),
            "parallelism": f"meshes sharded over {world} GPU(s) by size, no collective",
            "l2": "inputs larger than L2 (1.3 GB of triangles), no flush needed",
            "tuning": {"sort_digit_bits": int(tuning.sort_digit_bits), "sort_passes": passes,
                       "hploc_ctas_per_sm": int(tuning.hploc_ctas_per_sm),
                       "fusion_groups": int(tuning.fusion_groups), "block_size": int(tuning.block_size),
                       "fusion_point": fusion,
                       "candidates": int(tuning.candidates_tried), "tune_s": round(t_tune, 2)},
            "bvh8_nodes": int(n8),
            "loop_plain_api_ms": _num(t_loop * 1e3),
            "loop_plain_api_mtris_s": _num(n / t_loop / 1e6),
            "loop_async_ms": _num(t_loop_async * 1e3),
            "speedup_vs_loop_plain_api": _num(t_loop * 1e3 / ms),
            "speedup_vs_loop_async": _num(t_loop_async * 1e3 / ms),
        },
        "roofline": {"kernel": "whole batched pipeline", "bound": "hbm", "achieved": round(gbs, 1),
                     "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": round(gbs / pk["hbm_gbs"], 3), "traffic": None,
                     "peak_source": pk["source"]},
        "e2e": {"value": round(e2e_value, 2), "unit": "Mtris/s", "h2d_bytes_per_step": 36 * n,
                "d2h_bytes_per_step": 52 * meshes + 4,
                "call": "nxb_batch_build (graph replay + wait + per-mesh results) after a pinned host->device copy"},
        # per build: tile ranges, bounds, Morton, the sort passes, BVH8 queue
        # init, H-PLOC, BVH8, finalize (one mesh group)
        "gpu_launches": (7 + passes) * args.steps,
        "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline:
        import oracle
        oracle.set_level_collapse(True)
        t = time.perf_counter()
        done = 0
        m = 0
        while done < args.cpu_sample and m < meshes:
            k = int(counts[m])
            if k:
                r = oracle.build(np.ascontiguousarray(prims_np[off[m]:off[m + 1]]), 30, args.radius)
                assert r["err"] == 0
                done += k
            m += 1
        dt = time.perf_counter() - t
        line["cpu_baseline"] = {"value": round(done / dt / 1e6, 3), "unit": "Mtris/s", "cores": oracle.threads(),
                                "kind": "port", "sample": f"the first {m} meshes ({done:,} triangles), one CPU build "
                                                          f"each, in {dt:.2f} s"}
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


def run_served(args, world, rank, local):
    """Served form: a build server (nxb_server_*) fed Poisson arrivals; per
    request latency = submit -> completion, p50/p99 over the timed requests."""
    import threading
    import torch
    import nexusbvh_gb300 as nxb
    from nexusbvh_gb300 import scenes

    torch.cuda.set_device(local)
    nxb.load()
    pools = [scenes.uniform_soup(4_194_304, seed=0), scenes.displaced_sphere(2048, 1024, seed=1),
             scenes.clustered(4_194_304, seed=2), scenes.clustered(28_311_552, seed=5)]
    host = [torch.from_numpy(p).pin_memory() for p in pools]
    dev = [t.cuda() for t in host]
    total = args.warmup + args.steps
    reqs = served_requests(total)
    rate = 200.0
    rng = np.random.default_rng(12)
    gaps = rng.exponential(1.0 / rate, size=total)

    def run_pass(on_device: bool):
        srv = nxb.Server(budget_bytes=32 << 30, reserve=True)
        lat, queue, batched = [], [], 0
        tickets = []
        done = threading.Event()

        def drain():
            nonlocal batched
            for i, t in enumerate(iter(tickets_q.get, None)):
                r = srv.wait(t)
                if i >= args.warmup:
                    lat.append(r.latency_ms)
                    queue.append(r.queue_ms)
                    batched += r.batched_with > 1
                srv.release(t)
            done.set()

        import queue as _q
        tickets_q = _q.Queue()
        th = threading.Thread(target=drain)
        th.start()
        t0 = time.perf_counter()
        at = t0
        start_timed = None
        for i, (kind, n, kb) in enumerate(reqs):
            at += gaps[i]
            wait = at - time.perf_counter()
            if wait > 0.0005:
                time.sleep(wait - 0.0003)  # leave the GIL to the draining thread
            while time.perf_counter() < at:
                pass
            if i == args.warmup:
                start_timed = time.perf_counter()
            src = (dev if on_device else host)[kind][:n]
            cfg = nxb.BuildConfig(prioritize_speed=kb == 30)
            if on_device:
                t = srv.submit(src, cfg)
            else:
                t = srv.submit(src.numpy(), cfg)
            tickets.append(t)
            tickets_q.put(t)
        tickets_q.put(None)
        th.join()
        wall = time.perf_counter() - (start_timed or t0)
        st = srv.stats()
        srv.close()
        tris = sum(n for _, n, _ in reqs[args.warmup:])
        return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "mean_ms": float(np.mean(lat)), "max_ms": float(np.max(lat)),
                "queue_p99_ms": float(np.percentile(queue, 99)), "requests": len(lat),
                "batched_requests": batched, "wall_s": wall, "mtris_s": tris / wall / 1e6,
                "peak_bytes": int(st.peak_bytes_in_use), "builds": int(st.builds),
                "batched_builds": int(st.batched_builds)}

    def run_serial():
        """The same arrivals served by serial plain builds (the reference's
        model: one nxb_build_bvh8 call at a time, device-resident input)."""
        lib = nxb.load()
        out = nxb.CBVH8()
        stream_ptr = int(torch.cuda.current_stream().cuda_stream)
        lat = []
        t0 = time.perf_counter()
        at = t0
        arrivals = []
        for g in gaps:
            at += g
            arrivals.append(at)
        for i, (kind, n, kb) in enumerate(reqs):
            while time.perf_counter() < arrivals[i]:
                pass
            c = nxb.BuildConfig(prioritize_speed=kb == 30).to_c()
            nxb.check(lib.nxb_build_bvh8(dev[kind].data_ptr(), nxb.NXB_PRIM_TRIANGLE, n, ctypes.byref(c),
                                         stream_ptr, ctypes.byref(out), None), "nxb_build_bvh8")
            nxb.check(lib.nxb_free_device_bvh8(ctypes.byref(out)), "nxb_free_device_bvh8")
            if i >= args.warmup:
                lat.append((time.perf_counter() - arrivals[i]) * 1e3)
        return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "mean_ms": float(np.mean(lat)), "max_ms": float(np.max(lat))}

    with ClockSampler(local) as clocks:
        resident = run_pass(True)
        hostin = run_pass(False)
        serial = run_serial()
    if rank != 0:
        return
    n_big = sum(1 for k, _, _ in reqs[args.warmup:] if k == 3)
    line = {
        "metric": "p99 request latency, served builds (submit -> BVH8 done)",
        "value": round(resident["p99_ms"], 3), "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(resident["mean_ms"], 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generators standing in for the reference's scene files)",
        "config": {"workload": WORKLOADS["served"][0], "requests": args.steps, "big_requests": n_big,
                   "budget_gib": 32, "streams": 4, "batch_max_prims": 65536,
                   "l2": "each request's input is streamed once; the big builds exceed L2",
                   "device_resident": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in resident.items()},
                   "host_input": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in hostin.items()},
                   "serial_plain_builds": {k: round(v, 3) for k, v in serial.items()}},
        "roofline": None,
        "e2e": {"value": round(hostin["p99_ms"], 3), "unit": "ms",
                "h2d_bytes_per_step": int(np.mean([n * 36 for _, n, _ in reqs[args.warmup:]])),
                "d2h_bytes_per_step": 40,
                "call": "nxb_server_submit with host (pinned) input, nxb_server_wait, nxb_server_release"},
        "gpu_launches": None,
        "clocks": clocks.summary(),
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
    of a bounded prefix sample of the workload."""
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
        # a prefix of whole meshes, each built on its own
        last = int(np.searchsorted(off, min(args.cpu_sample, off[-1]), side="left"))
        last = max(1, min(last, meshes))
        subs = [np.ascontiguousarray(prims_np[off[i]:off[i + 1]]) for i in range(last) if counts[i]]
    else:
        prims_np = make_prims(args.workload)
        subs = [np.ascontiguousarray(prims_np[:min(args.cpu_sample, prims_np.shape[0])])]
    n = prims_np.shape[0]
    m = sum(x.shape[0] for x in subs)
    sub = subs[0]
    for _ in range(args.warmup):
        oracle.build(sub[: min(sub.shape[0], 65536)], key_bits, args.radius)
    times = []
    stage = np.zeros(5)
    for _ in range(args.steps):
        t = time.perf_counter()
        for x in subs:
            r = oracle.build(x, key_bits, args.radius)
            assert r["err"] == 0
            stage += np.array(r["stage_ms"])
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
                             "sample": f"first {m:,} of the workload's {n:,} triangles per step, one full CPU build "
                                       "(bounds, Morton, radix sort, H-PLOC, BVH8)",
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
    ap.add_argument("--cpu-sample", type=int, default=2_000_000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-loop-baseline", action="store_true",
                    help="batched workloads: leave out the loop-of-plain-builds comparison")
    ap.add_argument("--no-autotune", action="store_true",
                    help="batched workloads: build with the default tuning instead of tuning first")
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
