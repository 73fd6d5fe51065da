#!/usr/bin/env python3
"""Benchmark of the GB300 shadow hot path: DAG build + visibility lookups.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config c1|c0]

A step is one full build of the compressed shadow of the workload's depth
map (min-max pyramid, SVO classification with 64-bit leafmasks, subtree
merge, pointer compression), from a depth map resident in HBM to a DAG
resident in HBM.  `value` is whole-job build throughput in Gvoxel/s
(n^3 voxels per DAG).  `lookup` reports the workload's query batch against
the built DAG (Glookups/s).  `e2e` repeats both through the public API with
host buffers: the depth map / queries copied in from pinned host memory and
the DAG words / visibility bits read back, inside the timed region.

With --gpus N > 1 (under torchrun) every rank builds its own copy of the
workload (independent shadows, no collective on the data path: weak scaling)
and the slowest rank's time counts.  `--impl reference` times the CPU
restatement of the reference's own build and lookup (oracle/) on the host
cores instead.  Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from cpvs_gb300 import scene  # noqa: E402

WORKLOADS = {
    "c1": dict(queries=1 << 26, desc="8192^2 float32 depth map (plane 0.95, 500 boxes, 64 spheres; seed 1) -> "
                                      "8192^3-voxel DAG with 64-bit leafmasks; 2^26 float32 NDC lookups, half on "
                                      "the depth surface +-0.5 voxel, half uniform"),
    "c0": dict(queries=1 << 20, desc="1024^2 float32 depth map (plane 0.9, 40 boxes; seed 0) -> 1024^3-voxel DAG "
                                     "with 64-bit leafmasks; 2^20 NDC lookups"),
    "c2": dict(queries=1 << 27, desc="32768^2 float32 depth map (plane 0.95, 4000 boxes, 512 spheres; seed 2) in 8x8 "
                                      "xy tiles of 4096^2, 8 z-tiles each: 512 DAGs of 4096^3 in one grid build; 2^27 "
                                      "NDC lookups routed through the 8^3 grid"),
    "c4": dict(queries=0, desc="serving: Poisson arrivals, 1 build per 20 lookup batches; builds of config-0-style "
                                 "scenes (plane 0.9, 40 boxes) with sides 2^round(U[9,13]); lookup batches of "
                                 "2^round(U[12,22]) NDC points against a uniformly chosen resident DAG; 120 GB budget, "
                                 "LRU eviction; offered loads 0.8 and 1.5 of the serial plain path's capacity"),
    "c3": dict(queries=1 << 24, desc="64 independent lights (seeds 100..163, 10..2000 boxes, sides 2^round(U[8,13])) "
                                      "built in one batch; 2^24 NDC lookups spread over the 64 DAGs"),
}
METRIC = "DAG-build Gvoxel/s (shadow DAG from a depth map, bit-exact with the reference)"
CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms."""

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="cpvs_clocks_", suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={CLOCK_FIELDS}", "--format=csv,noheader,nounits", "-lms", "50",
                 "-i", str(self.device)], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append(dict(sm=float(f[1]), smax=float(f[2]), power=float(f[3]) if f[3] not in ("", "[N/A]") else 0.0,
                                 hw=f[5], hwt=f[6], swt=f[7], swp=f[8]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        pmax = max(r["power"] for r in rows)
        load = [r for r in rows if r["power"] >= 0.3 * pmax] or rows
        reasons = []
        for key, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"), ("swt", "sw_thermal_slowdown"),
                          ("swp", "sw_power_cap")):
            if any(r[key].lower() == "active" for r in load):
                reasons.append(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in load), "sm_max_mhz": max(r["smax"] for r in rows),
                "reasons": reasons, "samples": len(rows), "samples_under_load": len(load),
                "power_w_max": pmax}


# Algorithmic (minimum DRAM) bytes per kernel of one build: every input read
# once and every output written once; reads that the kernel repeats from
# cache (a depth texel shared by the leaves above it, a hot hash slot) count
# once.  These divide the kernel's CUDA-event time for `roofline.achieved`.
def kernel_alg_bytes(name: str, n: int, tree: list, uniq: list, dag_words: int, fused_leaves: bool = False) -> float:
    """Algorithmic bytes of one build's launches of kernel `name`.  With
    `fused_leaves` (no k_leaf_resolve launch: the expansion of level 3 looks
    each leaf's class up as it writes the leaf) the expansion also reads
    every column's 32-byte record once and writes job, class id and class
    mask per leaf (12 B, as many as the coordinate and job it no longer
    writes)."""
    leaves = tree[2] if len(tree) > 2 else 0
    # a build with leafmasks stores pyramid levels 3 and up (levels 1-2 stay on chip)
    first = 3 if leaves else 1
    texels = sum((n >> L) ** 2 for L in range(first, int(np.log2(n)) + 1))
    inner = sum(tree[3:])
    uleaves = uniq[2] if len(uniq) > 2 else 0
    cols = (n // 8) ** 2
    if name == "k_pyramid64":      # depth read once, every stored pyramid texel written once
        return 4.0 * n * n + 8.0 * texels
    if name == "k_leaf_columns":   # depth map once, the level-3 bounds once, a record per column; per leaf
        # class its masks, job and record (the 16 B run entries, one or more per column, are not counted)
        return 4.0 * n * n + cols * (8 + 8) + uleaves * (64 + 4 + 8)
    if name == "k_leaf_resolve":   # per leaf coord + job in, class id + class mask out; each column's
        # record once
        return leaves * (8 + 4 + 4 + 4) + cols * 8
    if name == "k_expand":         # per inner node coord + job + 2x2 pyramid texels in, mask + first out;
        # 12 B per child written
        return inner * (8 + 4 + 32 + 8) + (leaves + inner) * 12 + (cols * 32 if fused_leaves else 0)
    if name == "k_dedup_insert":   # per inner node mask + job + first + slot probe + slot out; 4 B per child id
        return inner * (4 + 4 + 4 + 8 + 4) + (leaves + inner) * 4
    if name == "k_merge_scan":     # per node slot + mask + job + table entry in; rank, offset out
        return (leaves + inner) * (4 + 4 + 4 + 8 + 4)
    if name == "k_emit_all":
        return 4.0 * dag_words
    return 0.0


def config_dict(config: str, n: int, dag_words: int, nq: int, world: int) -> dict:
    """The workload description both arms print (GPU and reference)."""
    wl = WORKLOADS[config]
    return {"workload": f"{config}: {wl['desc']}", "map_side": n, "voxels_per_dag": n ** 3,
            "dag_words": int(dag_words), "lookups_per_batch": nq,
            "l2": "inputs larger than L2 (256 MiB map read per step)" if n >= 8192 else
                  "map smaller than L2: later steps may hit L2",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}


def slowest_rank(torch, values, world: int, device) -> list:
    """Each per-rank time's maximum over the ranks: the job takes as long as
    its slowest replica."""
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return t.tolist()


def whole_job_rate(world: int, units_per_rank: float, ms: float) -> float:
    """Billions of units per second for the whole job: every replica
    processes `units_per_rank` per step, in `ms` of the slowest rank."""
    return world * units_per_rank / (ms * 1e-3) / 1e9


def host_link(torch, dev, stream, nbytes=256 << 20, reps=5) -> dict:
    """Copy rate of the host link: pinned host <-> device, one
    cudaMemcpyAsync of 256 MiB per direction, best of `reps` (CUDA events)."""
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    out = {}
    for name, dst, src in (("h2d_gbs", d, h), ("d2h_gbs", h, d)):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize(dev)
        best = 1e30
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            dst.copy_(src, non_blocking=True)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            best = min(best, e0.elapsed_time(e1))
        out[name] = round(nbytes / (best * 1e-3) / 1e9, 1)
    out["how"] = "one pinned cudaMemcpyAsync of 256 MiB per direction, best of 5, CUDA events"
    return out


def run_ours(args, rank, world, local_rank):
    import torch
    import cpvs_gb300 as cp

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    wl = WORKLOADS[args.config]
    sc = scene.config_scene(args.config)
    n = sc.n
    depth = scene.rasterise(sc)
    depth_pinned = torch.from_numpy(depth).pin_memory()
    depth_dev = depth_pinned.to(dev)
    nq = wl["queries"]
    q_host = scene.ndc_queries_mixed(depth, nq, 1)
    q_pinned = torch.from_numpy(q_host).pin_memory()
    q_dev = q_pinned.to(dev)
    bits_dev = torch.empty((nq + 31) // 32, dtype=torch.int32, device=dev)
    bits_host = torch.empty((nq + 31) // 32, dtype=torch.int32).pin_memory()

    ctx = cp.Context(local_rank)
    if args.fixed_shapes:
        # profiling aid: the default launch shapes, no tuning replays
        ctx.set_option(ctx.OPT_BUILD_CLUSTER_CAP, 8192)
        ctx.set_option(ctx.OPT_BUILD_INSERT_WAVES, 1)
    stream = torch.cuda.current_stream(dev)
    keep = {}

    def build_step():
        # CompressedShadow::create(const ShadowMap*) shape: hierarchy (reading
        # the resident map in place) + build in one call
        sh = cp.CompressedShadow.from_depth(depth_dev, ctx=ctx, stream=stream)
        keep["sh"] = sh  # the previous step's DAG is freed as this one replaces it
        return sh

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    if args.part in ("grid", "multi", "serve", "raster", "batch"):
        profile_part(args.part, cp, torch, ctx, dev, stream, args.warmup + args.steps)
        return
    if args.part == "frame":
        # profiling aid: the 4K frame (evaluate + shade) alone
        fr = measure_frame(cp, torch, ctx, build_step(), q_dev, stream, args.steps, args.warmup, barrier)
        print(json.dumps({"part": "frame", "ms_per_frame": fr["ms_per_frame"]}), flush=True)
        return
    if args.part != "all":
        # profiling aid: the build steps or the lookup batches alone
        sh = build_step()
        for _ in range(args.warmup + args.steps):
            if args.part == "build":
                build_step()
            else:
                sh.lookup_ndc(q_dev, bits_dev, stream=stream)
        torch.cuda.synchronize(dev)
        print(json.dumps({"part": args.part, "steps": args.warmup + args.steps}), flush=True)
        return

    clocks = ClockSampler(local_rank)
    clocks.start()
    # the SM clock takes a few hundred ms of load to ramp up from idle: build
    # for about a second before the counted warm-up steps, back to back as in
    # the timed region (each build waits for its own results inside the call)
    t_ramp = time.perf_counter()
    while time.perf_counter() - t_ramp < 1.0:
        build_step()
    torch.cuda.synchronize(dev)
    for _ in range(args.warmup):
        build_step()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        build_step()
    e1.record(stream)
    barrier()
    build_ms = e0.elapsed_time(e1) / args.steps
    # per-kernel CUDA-event timing: the same steps again with the library's
    # instrumentation on (every launch bracketed by events, launched eagerly)
    ctx.enable_timing(True)
    for _ in range(args.steps):
        build_step()
    barrier()
    ktimes = ctx.kernel_times()
    ctx.enable_timing(False)
    sh = keep["sh"]
    tree, uniq = sh.level_counts()
    dag_words = sh.dag_size()
    # the library's record of the last graph build: its internal-check word
    # must be 0 (any other bit fails the build), plus its re-plans and the
    # launch shapes the plan's tuner kept
    build_step()
    report = ctx.last_build()
    assert report["error_word"] == 0, report

    # lookups against the resident DAG, queries resident in HBM
    for _ in range(args.warmup):
        sh.lookup_ndc(q_dev, bits_dev, stream=stream)
    barrier()
    ctx.enable_timing(True)
    e0.record(stream)
    for _ in range(args.steps):
        sh.lookup_ndc(q_dev, bits_dev, stream=stream)
    e1.record(stream)
    barrier()
    lookup_ms = e0.elapsed_time(e1) / args.steps
    lk = ctx.kernel_times()["k_lookup"]
    ctx.enable_timing(False)
    # the tuner's alternatives (queries carried per thread), for the record
    variants = {}
    for qpt in (1, 2, 4):
        ctx.set_option(ctx.OPT_LOOKUP_QUERIES_PER_THREAD, qpt)
        sh.lookup_ndc(q_dev, bits_dev, stream=stream)
        e0.record(stream)
        for _ in range(3):
            sh.lookup_ndc(q_dev, bits_dev, stream=stream)
        e1.record(stream)
        barrier()
        variants[str(qpt)] = round(e0.elapsed_time(e1) / 3, 4)
    ctx.set_option(ctx.OPT_LOOKUP_QUERIES_PER_THREAD, 0)
    # a build followed by its first lookup batch, the serving pattern: the
    # first lookup also builds the DAG's top grid (k_top_index)
    first = []
    ctx.enable_timing(True)
    for _ in range(3):
        e0.record(stream)
        s2 = cp.CompressedShadow.from_depth(depth_dev, ctx=ctx, stream=stream)
        s2.lookup_ndc(q_dev, bits_dev, stream=stream)
        e1.record(stream)
        barrier()
        first.append(e0.elapsed_time(e1))
        del s2
    top_kt = ctx.kernel_times().get("k_top_index", (0.0, 0))
    ctx.enable_timing(False)

    # end to end through the public API with host buffers
    # the DAG is read back into one reused pinned buffer, as the lookup bits are
    dag_host = torch.empty(max(2 * keep["sh"].dag_size(), 1 << 20), dtype=torch.int32).pin_memory()

    def e2e_build():
        s = cp.CompressedShadow.from_depth(depth_pinned, ctx=ctx, stream=stream)
        s.get_dag(out=dag_host, stream=stream)
        return s
    for _ in range(max(1, args.warmup // 2)):
        e2e_build()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s = e2e_build()
    barrier()
    e2e_build_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    dag_bytes = s.dag_size() * 4
    del s
    for _ in range(max(1, args.warmup // 2)):
        sh.lookup_ndc_packed(q_pinned, bits_host, stream=stream)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sh.lookup_ndc_packed(q_pinned, bits_host, stream=stream)
    barrier()
    e2e_lookup_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    # one rendered frame against this DAG (4K G-buffer; needs that many lookup points)
    frame = (measure_frame(cp, torch, ctx, sh, q_dev, stream, args.steps, args.warmup, barrier)
             if world == 1 and nq >= 3840 * 2160 else None)
    clk = clocks.stop()
    link = host_link(torch, dev, stream) if world == 1 else None

    # slowest rank
    build_ms, lookup_ms, e2e_build_ms, e2e_lookup_ms = slowest_rank(
        torch, [build_ms, lookup_ms, e2e_build_ms, e2e_lookup_ms], world, dev)
    voxels = float(n) ** 3

    # kernels launched in the timed region: the eager pass's timing scopes,
    # each counted by the kernels it wraps (the pyramid scope one per pass,
    # the leaf-column scope its two passes, the table clear a memset), plus
    # the one k_clear of every build (launched without a scope)
    kernels_per_scope = {"k_pyramid64": -(-int(np.log2(n)) // 6), "k_leaf_columns": 2, "table_clear": 0}
    timed_launches = sum(v[1] * kernels_per_scope.get(k, 1) for k, v in ktimes.items()) + args.steps
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    peak, peak_kind = peaks()
    build_kernels = {k: v for k, v in ktimes.items() if v[1] and k not in ("k_lookup", "k_grid_lookup")}
    dom = max(build_kernels, key=lambda k: build_kernels[k][0])
    dom_ms_launch = build_kernels[dom][0] / build_kernels[dom][1]
    dom_launches_per_step = build_kernels[dom][1] / args.steps
    fused_leaves = "k_leaf_resolve" not in build_kernels
    dom_bytes = kernel_alg_bytes(dom, n, tree, uniq, dag_words, fused_leaves) / dom_launches_per_step
    achieved = dom_bytes / (dom_ms_launch * 1e-3) / 1e9
    # DRAM bytes per launch from the committed ncu launch list of this
    # workload (profiles/traffic_<config>.json), when it has one
    prof = os.path.join(ROOT, "profiles", f"traffic_{args.config}.json")
    measured = json.load(open(prof)) if os.path.exists(prof) else {}
    # the lookup kernel's DRAM and L2 figures from its committed ncu capture
    # (profiles/lookup_<config>.json), when this workload has one
    lk_prof_path = os.path.join(ROOT, "profiles", f"lookup_{args.config}.json")
    lk_prof = json.load(open(lk_prof_path)) if os.path.exists(lk_prof_path) else {}

    def traffic_of(k):
        t = measured.get(k)
        return int(t["dram_bytes_per_build"] / max(t["launches_per_build"], 1)) if isinstance(t, dict) else None
    traffic = traffic_of(dom)
    # every build kernel's roofline on its own algorithmic bytes
    kernel_rooflines = {}
    for k, (tot_ms, launches) in build_kernels.items():
        per = launches / args.steps
        alg = kernel_alg_bytes(k, n, tree, uniq, dag_words, fused_leaves)
        if not alg or not per:
            continue
        ms_l = tot_ms / launches
        ach = alg / per / (ms_l * 1e-3) / 1e9
        kernel_rooflines[k] = {"launches_per_step": round(per, 2), "ms_per_launch": round(ms_l, 4),
                               "alg_bytes_per_launch": int(alg / per), "achieved_gbs": round(ach, 1),
                               "frac": round(ach / peak, 4), "traffic_per_launch": traffic_of(k)}
    # the map once, the stored pyramid levels (3 and up for a leafmask build) once, the DAG once
    build_alg = 4.0 * n * n + 8.0 * sum((n >> L) ** 2 for L in range(3, int(np.log2(n)) + 1)) + 4.0 * dag_words
    build_alg_all = 4.0 * n * n + 16.0 * n * n / 3.0 + 4.0 * dag_words
    lookup_alg = nq * 12.125 + 4.0 * dag_words
    lk_ms_launch = lk[0] / max(lk[1], 1)
    line = {
        "metric": METRIC,
        "value": round(whole_job_rate(world, voxels, build_ms), 1),
        "unit": "Gvoxel/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(build_ms, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic: seeded scene rasterised to a float32 depth map (no dataset involved)",
        "config": config_dict(args.config, n, dag_words, nq, world),
        "e2e": {"value": round(whole_job_rate(world, voxels, e2e_build_ms), 1), "unit": "Gvoxel/s",
                "h2d_bytes_per_step": int(depth.nbytes), "d2h_bytes_per_step": int(dag_bytes),
                "ms_per_step": round(e2e_build_ms, 3),
                "path": "cpvs_shadow_create_from_depth (pinned host map) + cpvs_shadow_dag_words (into pinned host memory)"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind, "traffic": traffic,
                     "alg_bytes_per_launch": int(dom_bytes), "ms_per_launch": round(dom_ms_launch, 4),
                     "build_pipeline": {"alg_bytes": int(build_alg),
                                        "achieved": round(build_alg / (build_ms * 1e-3) / 1e9, 1),
                                        "frac": round(build_alg / (build_ms * 1e-3) / 1e9 / peak, 4),
                                        # the byte model with every pyramid level written
                                        # and read once (4n^2 + 16n^2/3 + 4 |DAG|)
                                        "all_levels_model": {
                                            "alg_bytes": int(build_alg_all),
                                            "frac": round(build_alg_all / (build_ms * 1e-3) / 1e9 / peak, 4)}}},
        "lookup": {"value": round(whole_job_rate(world, nq, lookup_ms), 2), "unit": "Glookups/s",
                   "ms_per_batch": round(lookup_ms, 4), "ms_by_queries_per_thread": variants,
                   "roofline": {"bound": "hbm", "achieved": round(lookup_alg / (lk_ms_launch * 1e-3) / 1e9, 1),
                                "peak": peak, "unit": "GB/s",
                                "frac": round(lookup_alg / (lk_ms_launch * 1e-3) / 1e9 / peak, 4),
                                "alg_bytes_per_launch": int(lookup_alg),
                                "traffic": lk_prof.get("dram_bytes_per_launch"),
                                "l2_throughput_frac_ncu": lk_prof.get("l2_throughput_frac"),
                                "l2_hit_rate_ncu": lk_prof.get("l2_hit_rate")},
                   "e2e": {"value": round(whole_job_rate(world, nq, e2e_lookup_ms), 2), "unit": "Glookups/s",
                           "h2d_bytes_per_step": int(q_host.nbytes), "d2h_bytes_per_step": int(bits_host.numel() * 4),
                           "ms_per_step": round(e2e_lookup_ms, 3)}},
        "build_then_first_lookup": {"ms": round(statistics.median(first), 4),
                                    "steady_build_plus_lookup_ms": round(build_ms + lookup_ms, 4),
                                    "k_top_index_ms": round(top_kt[0] / max(top_kt[1], 1), 4),
                                    "path": "cpvs_shadow_create_from_depth, then the first cpvs_shadow_lookup_ndc "
                                            "on the new shadow (builds its top grid), median of 3"},
        "build_report": report,
        "kernel_rooflines": kernel_rooflines,
        "kernels_ms_per_step": {k: round(v[0] / args.steps, 4) for k, v in build_kernels.items()},
        "kernel_timing": "CUDA events around every library launch, in a pass of the same steps right after the "
                         "timed region (the timed region itself replays the captured build graph)",
        "gpu_launches": int(timed_launches),
        "clocks": clk,
    }
    if link is not None:
        # end to end against the host link: the bytes each step moves across
        # it, at the link's measured copy rate, bound the step from below
        def link_roofline(h2d, d2h, ms):
            floor = (h2d / (link["h2d_gbs"] * 1e9) + d2h / (link["d2h_gbs"] * 1e9)) * 1e3
            return {"bound": "host link", "floor_ms": round(floor, 4), "frac": round(floor / ms, 4),
                    "achieved_gbs": round((h2d + d2h) / (ms * 1e-3) / 1e9, 1)}
        line["host_link"] = link
        line["e2e"]["roofline"] = link_roofline(depth.nbytes, dag_bytes, e2e_build_ms)
        line["lookup"]["e2e"]["roofline"] = link_roofline(q_host.nbytes, bits_host.numel() * 4, e2e_lookup_ms)
    if frame is not None:
        fr = frame["shade_roofline"]
        fr.update({"peak": peak, "unit": "GB/s", "frac": round(fr["achieved"] / peak, 4), "peak_kind": peak_kind})
        line["frame"] = frame
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(depth, q_host, args.config, sample_queries=1 << 22)
    if world == 1 and not args.no_extras:
        # the batched and served forms on the same GPU, each against the
        # plain per-request path (their own clocks; not part of `value`)
        drop = ("n_gpus", "higher_is_better", "scaling", "vs_baseline", "dtype", "data")
        del q_dev, bits_dev, depth_dev
        keep.clear()
        torch.cuda.empty_cache()
        xs = min(args.steps, 10)
        for key, cfg in (("batched", "c3"), ("grid", "c2")):
            r = measure_batched(cfg, xs, 3, cpu=not args.no_cpu_baseline)
            line[key] = {k: v for k, v in r.items() if k not in drop}
            torch.cuda.empty_cache()
        r = measure_served()
        line["served"] = {k: v for k, v in r.items() if k not in drop}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def profile_part(part, cp, torch, ctx, dev, stream, reps):
    """Profiling aids for the kernels outside the c1 build and lookup, on
    small cases (inputs above L2, a few GB on the device at most):
    grid   -- a 4x4 grid of 2048^2 xy tiles of the c2 scene, 4 z-tiles each
              (64 DAGs, one batched build), 2^24 NDC lookups routed through it
              (k_grid_top_index, k_grid_lookup);
    multi  -- 16 of the c3 lights in one batch, 2^24 points spread over them
              (k_top_index per DAG, k_multi_lookup);
    serve  -- 64 lookup requests of 2^18 points through a server holding 4
              DAGs, in one segmented launch each round (k_segment_lookup);
    raster -- the c1 scene rasterised to an 8192^2 depth map (k_raster);
    batch  -- 16 of the c3 lights' hierarchies in one batched call, then one
              batch build (k_zero_flags, k_pyramid_batch)."""
    gen = torch.Generator(device=dev)
    gen.manual_seed(11)
    if part == "raster":
        sc = scene.config_scene("c1")
        for _ in range(reps):
            cp.raster_depth(sc, ctx=ctx)
    elif part == "grid":
        sc = scene.config_scene("c2", n=8192)
        T, L = 2048, 4
        maps = [cp.raster_depth(sc, x * T, y * T, T, T, ctx=ctx) for y in range(L) for x in range(L)]
        hs = [cp.MinMaxHierarchy(m, ctx=ctx, stream=stream, borrow=True) for m in maps]
        grid = cp.CompressedShadowContainer(L, ctx=ctx)
        grid.build(hs, stream=stream)
        q = (torch.rand((1 << 24, 3), generator=gen, device=dev) * 2 - 1).contiguous()
        out = torch.empty((1 << 24) // 32, dtype=torch.int32, device=dev)
        for _ in range(reps):
            grid.lookup_ndc(q, out, stream=stream)
    elif part == "batch":
        # 16 of the c3 lights: their hierarchies in one batched call, then
        # one batch build
        maps = [cp.raster_depth(s, ctx=ctx) for s in c3_scenes()[:16]]
        for _ in range(reps):
            hs = cp.MinMaxHierarchy.create_batch(maps, ctx=ctx, stream=stream, borrow=True)
            cp.CompressedShadow.create_batch(hs, [(i, 0, 1) for i in range(len(hs))], stream=stream)
    elif part == "multi":
        scs = c3_scenes()[:16]
        maps = [cp.raster_depth(s, ctx=ctx) for s in scs]
        hs = [cp.MinMaxHierarchy(m, ctx=ctx, stream=stream, borrow=True) for m in maps]
        shs = cp.CompressedShadow.create_batch(hs, [(i, 0, 1) for i in range(len(hs))], stream=stream)
        ids = torch.randint(0, len(shs), (1 << 24,), generator=gen, device=dev, dtype=torch.int32)
        q = (torch.rand((1 << 24, 3), generator=gen, device=dev) * 2 - 1).contiguous()
        out = torch.empty((1 << 24) // 32, dtype=torch.int32, device=dev)
        for _ in range(reps):
            cp.lookup_ndc_multi(shs, ids, q, out, stream=stream)
    elif part == "serve":
        srv = cp.Server(cp.Context(dev.index or 0), budget_bytes=1 << 30)
        for key in range(4):
            d = scene.rasterise(scene.make_scene(2048, 0.9, 40, 0, 500 + key))
            srv.wait(srv.submit_build(key, torch.from_numpy(d).pin_memory()))
        pts = torch.from_numpy((np.random.default_rng(3).random((1 << 18, 3)) * 2 - 1).astype(np.float32)).pin_memory()
        for _ in range(reps):
            tickets = [srv.submit_lookup(k % 4, pts) for k in range(64)]
            for t in tickets:
                srv.wait(t, packed=True)
        srv.close()
    torch.cuda.synchronize(dev)
    print(json.dumps({"part": part, "reps": reps}), flush=True)


def measure_frame(cp, torch, ctx, sh, q_dev, stream, steps, warmup, barrier, width=3840, height=2160):
    """One frame of the reference's renderer after the precompute
    (DeferredRenderer::doAllShading): evaluate the DAG at every pixel of a
    3840x2160 rgba32f G-buffer, then the shading pass.  Light space is the
    world here (identity view-projection); the positions are the first
    8.3 M of the workload's lookup points, all on the depth surface (where a
    G-buffer's positions lie; each descends to a leaf) and in random order
    (a rendered frame's neighbouring pixels would be neighbouring voxels);
    the normals are random unit vectors and the albedo random.  The G-buffer
    (398 MB) is larger than L2."""
    dev = q_dev.device
    npix = width * height
    gen = torch.Generator(device=dev)
    gen.manual_seed(3)
    pos = torch.ones((height, width, 4), dtype=torch.float32, device=dev)
    pos[..., :3] = q_dev[:npix].reshape(height, width, 3)
    nrm = torch.randn((height, width, 4), generator=gen, device=dev)
    nrm[..., :3] /= nrm[..., :3].norm(dim=-1, keepdim=True)
    alb = torch.rand((height, width, 4), generator=gen, device=dev)
    out = torch.empty((height, width, 4), dtype=torch.float32, device=dev)
    vis = torch.empty((height, width), dtype=torch.uint8, device=dev)
    grid = cp.CompressedShadowContainer.of(sh)
    grid.copy_to_gpu(stream=stream)
    M = np.eye(4, dtype=np.float32)
    light = (0.3, 0.4, -1.0)

    def one():
        grid.evaluate(pos, M, out=vis, stream=stream)
        cp.shade(nrm, alb, light, visibilities=vis, out=out, ctx=ctx, stream=stream)
    for _ in range(warmup):
        one()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.enable_timing(True)
    e0.record(stream)
    for _ in range(steps):
        one()
    e1.record(stream)
    barrier()
    kt = ctx.kernel_times()
    ctx.enable_timing(False)
    frame_ms = e0.elapsed_time(e1) / steps
    ev, sd = kt["k_grid_evaluate"], kt["k_shade"]
    shade_ms = sd[0] / max(sd[1], 1)
    shade_bytes = npix * (16 + 16 + 1 + 16)  # normal, albedo, visibility byte in; colour out
    return {"pixels": npix, "resolution": f"{width}x{height}", "ms_per_frame": round(frame_ms, 4),
            "fps": round(1e3 / frame_ms, 1), "evaluate_ms": round(ev[0] / max(ev[1], 1), 4),
            "shade_ms": round(shade_ms, 4),
            "path": "cpvs_grid_evaluate (u8, filter 1) + cpvs_shade, G-buffer resident in HBM",
            "shade_roofline": {"bound": "hbm", "kernel": "k_shade", "alg_bytes_per_launch": shade_bytes,
                               "achieved": round(shade_bytes / (shade_ms * 1e-3) / 1e9, 1)},
            "gpu_launches": int(ev[1] + sd[1])}


def host_cpu() -> dict:
    """The host's core count and CPU model (lscpu's name where it has one)."""
    model = platform.processor() or platform.machine()
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().startswith("Model name:"):
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"nproc": os.cpu_count() or 1, "cpu": model, "arch": platform.machine()}


def cpu_parallel_builds(jobs, label):
    """Independent DAG builds of the CPU restatement, one per host core at a
    time (the oracle holds no shared state; its calls release the GIL), as
    the reference runs one create per thread over z-tiles.  `jobs`: (map,
    z_index, z_num).  Returns the bounded-sample CPU baseline."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle.oracle import Oracle
    O = Oracle()
    workers = min(os.cpu_count() or 1, len(jobs))
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=workers) as ex:
        list(ex.map(lambda j: O.build(j[0], j[1], j[2], threads=1), jobs))
    wall = time.perf_counter() - t0
    voxels = sum(float(j[0].shape[0]) ** 3 for j in jobs)  # a z-tile DAG covers N^3 voxels too
    return {"value": round(voxels / wall / 1e9, 3), "unit": "Gvoxel/s", "cores": workers, "kind": "port",
            "sample": f"{len(jobs)} DAG builds ({label}) on {workers} threads, {wall:.2f} s wall",
            "host": host_cpu()}


def cpu_baseline(depth, q, config, sample_queries, threads=None):
    """The CPU restatement of the reference's build (pyramid on 4 threads as
    the reference splits it, create on one thread as the reference runs it)
    and its lookups on every host core."""
    from oracle.oracle import Oracle
    O = Oracle()
    threads = threads or os.cpu_count() or 1
    n = depth.shape[0]
    t0 = time.perf_counter()
    b = O.build(depth, threads=4)
    build_s = time.perf_counter() - t0
    qs = np.ascontiguousarray(q[:sample_queries])
    t0 = time.perf_counter()
    O.lookup_ndc(b.dag, b.num_levels, b.leafmasks, qs, threads=threads)
    look_s = time.perf_counter() - t0
    q1 = np.ascontiguousarray(q[:1 << 20])
    t0 = time.perf_counter()
    O.lookup_ndc(b.dag, b.num_levels, b.leafmasks, q1, threads=1)
    look1_s = time.perf_counter() - t0
    return {"value": round(float(n) ** 3 / build_s / 1e9, 3), "unit": "Gvoxel/s", "cores": 4, "kind": "port",
            "sample": f"one full {config} build ({n}^2 map, pyramid on 4 threads, SVO/merge/compress on 1 thread, "
                      f"{build_s:.2f} s); hash-indexed first-occurrence merge (the reference's linear scan gives "
                      f"the same DAG more slowly)",
            "lookup": {"value": round(qs.shape[0] / look_s / 1e9, 4), "unit": "Glookups/s", "cores": threads,
                       "sample": f"{qs.shape[0]} of the {config} queries",
                       "one_core": {"value": round(q1.shape[0] / look1_s / 1e9, 4), "unit": "Glookups/s",
                                    "sample": f"{q1.shape[0]} queries on 1 thread"}},
            "host": host_cpu()}


def run_reference(args, rank, world):
    if rank != 0:
        return
    wl = WORKLOADS[args.config]
    sc = scene.config_scene(args.config)
    n = sc.n
    depth = scene.rasterise(sc)
    q = scene.ndc_queries_mixed(depth, wl["queries"], 1)
    from oracle.oracle import Oracle
    O = Oracle()
    threads = os.cpu_count() or 1
    # each step: one full build (the reference builds one DAG per thread) plus
    # one bounded lookup sample over all host cores; --steps and --warmup as
    # given (20 and 5 builds of ~3 s each at 8192^2 take about 75 s)
    steps = max(1, args.steps)
    warm = max(0, args.warmup)
    sample = min(wl["queries"], 1 << 23)
    for _ in range(warm):
        O.build(depth, threads=4)
    tb, tl = [], []
    b = None
    for _ in range(steps):
        t0 = time.perf_counter()
        b = O.build(depth, threads=4)
        tb.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        O.lookup_ndc(b.dag, b.num_levels, b.leafmasks, q[:sample], threads=threads)
        tl.append(time.perf_counter() - t0)
    build_s = statistics.mean(tb)
    v = float(n) ** 3 / build_s / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": "Gvoxel/s", "n_gpus": world,
        "steps": steps, "warmup": warm, "ms_per_step": round(build_s * 1e3, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded scene rasterised to a float32 depth map (no dataset involved)",
        "config": config_dict(args.config, n, int(b.dag.size), wl["queries"], world),
        "cpu_baseline": {"value": round(v, 3), "unit": "Gvoxel/s", "cores": 4, "kind": "port",
                         "sample": f"full {n}^2 build per step: pyramid on 4 threads, SVO/merge/compress on 1 thread "
                                   f"(the reference's threading); hash-indexed first-occurrence merge",
                         "host": host_cpu()},
        "e2e": {"value": round(v, 3), "unit": "Gvoxel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "lookup": {"value": round(sample / statistics.mean(tl) / 1e9, 4), "unit": "Glookups/s", "cores": threads,
                   "sample": f"{sample} queries per step"},
    }
    print(json.dumps(line), flush=True)


def c3_scenes():
    """64 lights: side 2^round(8 + 5u), 10 + floor(1991u) boxes, plane 0.9."""
    meta = scene.SplitMix64(3)
    out = []
    for i in range(64):
        side = 1 << int(round(8 + 5 * meta.uniform()))
        nb = 10 + int(1991 * meta.uniform())
        out.append(scene.make_scene(side, 0.9, nb, 0, 100 + i))
    return out


def surface_queries_device(torch, maps, n_total, count, gen, tile_of=None):
    """`count` NDC points on the depth surfaces of `maps` (device tensors),
    offset by up to half a voxel in z, at path resolution `n_total`."""
    k = len(maps)
    which = torch.randint(0, k, (count,), generator=gen, device=maps[0].device)
    out = torch.empty((count, 3), dtype=torch.float32, device=maps[0].device)
    scale = 2.0 / (n_total - 1)
    for i, m in enumerate(maps):
        sel = (which == i).nonzero().squeeze(1)
        if sel.numel() == 0:
            continue
        h, w = m.shape
        px = torch.randint(0, w, (sel.numel(),), generator=gen, device=m.device)
        py = torch.randint(0, h, (sel.numel(),), generator=gen, device=m.device)
        ox, oy, oz, nz = tile_of(i) if tile_of else (0, 0, 0, w)
        vz = m[py, px].double() * nz + (torch.rand(sel.numel(), generator=gen, device=m.device, dtype=torch.float64) - 0.5)
        out[sel, 0] = ((px + ox + 0.5) * scale - 1.0).float()
        out[sel, 1] = ((py + oy + 0.5) * scale - 1.0).float()
        out[sel, 2] = ((vz + oz) * scale - 1.0).float()
    return out, which


def measure_batched(config: str, steps: int, warmup: int, cpu: bool = True) -> dict:
    """c2 / c3: many DAGs per step in one batched build (one plan, one graph
    launch) against the plain path (one build call per DAG)."""
    import torch
    import cpvs_gb300 as cp
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    wl = WORKLOADS[config]
    ctx = cp.Context(0)
    stream = torch.cuda.current_stream(dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(7)
    nq = wl["queries"]
    if config == "c2":
        sc = scene.config_scene("c2")
        T, L = 4096, 8
        maps = [cp.raster_depth(sc, x * T, y * T, T, T, ctx=ctx) for y in range(L) for x in range(L)]
        voxels = float(T) ** 3 * L ** 3
        half = nq // 2
        qs, _ = surface_queries_device(torch, maps, T * L, half, gen,
                                       tile_of=lambda i: ((i % L) * T, (i // L) * T, 0, T * L))
        qu = torch.rand((nq - half, 3), generator=gen, device=dev) * 2 - 1
        q = torch.cat([qs, qu]).contiguous()

        def batched():
            # every tile's pyramid in one launch per pass, then one grid build
            hs = cp.MinMaxHierarchy.create_batch(maps, ctx=ctx, stream=stream, borrow=True)
            grid = cp.CompressedShadowContainer(L, ctx=ctx)
            grid.build(hs, stream=stream)
            return grid

        def plain():
            hs = [cp.MinMaxHierarchy(m, ctx=ctx, stream=stream, borrow=True) for m in maps]
            grid = cp.CompressedShadowContainer(L, ctx=ctx)
            for z in range(L):
                for y in range(L):
                    for x in range(L):
                        grid.set(cp.CompressedShadow.create(hs[y * L + x], z, L, stream=stream), x, y, z)
            grid.copy_to_gpu(stream=stream)
            return grid

        def look(g, out):
            return g.lookup_ndc(q, out, stream=stream)
        ndags = L ** 3
    else:
        scs = c3_scenes()
        maps = [cp.raster_depth(s, ctx=ctx) for s in scs]
        voxels = float(sum(s.n ** 3 for s in scs))
        half = nq // 2
        # surface points of each light at its own resolution, half uniform
        ids = torch.randint(0, len(maps), (nq,), generator=gen, device=dev, dtype=torch.int64)
        q = torch.rand((nq, 3), generator=gen, device=dev) * 2 - 1
        for i, m in enumerate(maps):
            sel = (ids[:half] == i).nonzero().squeeze(1)
            if sel.numel() == 0:
                continue
            nmap = m.shape[0]
            px = torch.randint(0, nmap, (sel.numel(),), generator=gen, device=dev)
            py = torch.randint(0, nmap, (sel.numel(),), generator=gen, device=dev)
            vz = m[py, px].double() * nmap + (torch.rand(sel.numel(), generator=gen, device=dev, dtype=torch.float64) - 0.5)
            sc2 = 2.0 / (nmap - 1)
            q[sel, 0] = ((px + 0.5) * sc2 - 1).float()
            q[sel, 1] = ((py + 0.5) * sc2 - 1).float()
            q[sel, 2] = (vz * sc2 - 1).float()
        ids32 = ids.to(torch.int32).contiguous()
        q = q.contiguous()

        def batched():
            # every light's pyramid in one launch per pass, then one batch build
            hs = cp.MinMaxHierarchy.create_batch(maps, ctx=ctx, stream=stream, borrow=True)
            return cp.CompressedShadow.create_batch(hs, [(i, 0, 1) for i in range(len(hs))], stream=stream)

        def plain():
            out = []
            for m in maps:
                h = cp.MinMaxHierarchy(m, ctx=ctx, stream=stream, borrow=True)
                out.append(cp.CompressedShadow.create(h, stream=stream))
            return out

        def look(shs, out):
            return cp.lookup_ndc_multi(shs, ids32, q, out, stream=stream)
        ndags = len(maps)
    out = torch.empty((nq + 31) // 32, dtype=torch.int32, device=dev)

    def timed(fn, steps, warm):
        keep = None
        for _ in range(warm):
            keep = fn()
        torch.cuda.synchronize()
        times = []
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            keep = fn()
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        return keep, times

    clocks = ClockSampler(0)
    clocks.start()
    res_b, tb = timed(batched, steps, warmup)
    res_p, tp = timed(plain, max(2, steps // 4), 1)
    # correctness of the batched form against the plain one on the same maps
    same = None
    if config == "c3":
        same = all(np.array_equal(a.get_dag(), b.get_dag()) for a, b in zip(res_b, res_p))
    else:
        da, _ = res_b.words()
        db, _ = res_p.words()
        same = bool(np.array_equal(da, db))
    for _ in range(3):
        look(res_b, out)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        look(res_b, out)
    e1.record(stream)
    torch.cuda.synchronize()
    look_ms = e0.elapsed_time(e1) / steps
    clk = clocks.stop()
    ms_b = statistics.median(tb)
    ms_p = statistics.median(tp)
    line = {
        "metric": METRIC + (" -- batched grid build" if config == "c2" else " -- batched multi-light build"),
        "value": round(voxels / (ms_b * 1e-3) / 1e9, 1), "unit": "Gvoxel/s", "n_gpus": 1, "steps": steps,
        "warmup": warmup, "ms_per_step": round(ms_b, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic: seeded scenes rasterised on the GPU (no dataset)",
        "config": {"workload": f"{config}: {wl['desc']}", "dags_per_step": ndags, "voxels_per_step": voxels},
        "plain": {"value": round(voxels / (ms_p * 1e-3) / 1e9, 1), "unit": "Gvoxel/s", "ms_per_step": round(ms_p, 3),
                  "path": "one cpvs_shadow_create per DAG" + (" + grid finalize" if config == "c2" else "")},
        "batched_over_plain": round(ms_p / ms_b, 2),
        "p50_ms": {"batched": round(ms_b, 3), "plain": round(ms_p, 3)},
        "p99_ms": {"batched": round(float(np.percentile(tb, 99)), 3), "plain": round(float(np.percentile(tp, 99)), 3)},
        "dags_identical_to_plain": same,
        "lookup": {"value": round(nq / (look_ms * 1e-3) / 1e9, 2), "unit": "Glookups/s", "ms_per_batch": round(look_ms, 4),
                   "path": "cpvs_grid_lookup_ndc" if config == "c2" else "cpvs_lookup_ndc_multi"},
        "clocks": clk,
    }
    if cpu:
        if config == "c2":
            # the 8 z-tile DAGs of the 8 xy tiles on the grid's diagonal (1/8 of the DAGs)
            diag = [t * (L + 1) for t in range(L)]
            jobs = [(maps[t].cpu().numpy(), z, L) for t in diag for z in range(L)]
            line["cpu_baseline"] = cpu_parallel_builds(jobs, "8 z-tiles of the 8 diagonal xy tiles of 4096^2")
        else:
            jobs = [(m.cpu().numpy(), 0, 1) for m in maps[:16]]
            line["cpu_baseline"] = cpu_parallel_builds(jobs, "the first 16 of the 64 lights")
    return line


def run_batched(args):
    print(json.dumps(measure_batched(args.config, args.steps, args.warmup, not args.no_cpu_baseline)), flush=True)


def measure_served() -> dict:
    """c4: the same request trace through the server (continuous batching)
    and through serial plain-path handling on the same GPU; then a trace
    whose lookups go to the 6 most recent builds through a server with a
    12 MiB budget (the trace builds ~16 MB of DAGs), so that older DAGs are
    evicted (LRU) and builds admitted by bytes."""
    import threading
    import torch
    import cpvs_gb300 as cp
    torch.cuda.set_device(0)
    ctx = cp.Context(0)
    sides = [512, 1024, 2048, 4096, 8192]
    pool = {}
    for si, side in enumerate(sides):
        for v in range(2):
            sc = scene.make_scene(side, 0.9, 40, 0, 400 + 10 * si + v)
            pool[(side, v)] = cp.raster_depth(sc, ctx=ctx).cpu().pin_memory()
    g = np.random.Generator(np.random.PCG64(44))
    pts_pool = torch.from_numpy((g.random((1 << 22, 3)) * 2 - 1).astype(np.float32)).pin_memory()
    meta = np.random.Generator(np.random.PCG64(45))
    nreq = 4000

    def make_trace(rate, recent=0):
        # recent > 0: lookups pick one of the `recent` latest builds
        t, trace, built = 0.0, [], []
        for i in range(nreq):
            t += meta.exponential(1.0 / rate)
            if not built or meta.random() < 1.0 / 21.0:
                side = 1 << int(round(9 + 4 * meta.random()))
                trace.append(("build", t, i, pool[(side, int(meta.integers(0, 2)))]))
                built.append(i)
            else:
                cnt = 1 << int(round(12 + 10 * meta.random()))
                off = int(meta.integers(0, pts_pool.shape[0] - cnt + 1))
                pick = built[-recent:] if recent else built
                trace.append(("lookup", t, pick[int(meta.integers(0, len(pick)))], pts_pool[off:off + cnt]))
        return trace

    def plain_run(trace):
        shadows, lat = {}, {"build": [], "lookup": []}
        t0 = time.perf_counter()
        for kind, at, key, data in trace:
            now = time.perf_counter() - t0
            if now < at:
                time.sleep(at - now)
            if kind == "build":
                shadows[key] = cp.CompressedShadow.from_depth(data, ctx=ctx)
            else:
                out = np.empty((data.shape[0] + 31) // 32, np.uint32)
                shadows[key].lookup_ndc_packed(data, out)
            lat[kind].append((time.perf_counter() - t0 - at) * 1e3)
        return lat, time.perf_counter() - t0

    def served_run(trace, budget=120 << 30):
        """The trace through the server; latency counts from the scheduled
        arrival (a late submission counts against the server)."""
        srv = cp.Server(cp.Context(0), budget_bytes=budget)
        tickets = []
        t0 = time.perf_counter()

        def submitter():
            for kind, at, key, data in trace:
                now = time.perf_counter() - t0
                if now < at:
                    time.sleep(at - now)
                late = (time.perf_counter() - t0 - at) * 1e3
                if kind == "build":
                    tickets.append((kind, late, srv.submit_build(key, data)))
                else:
                    out = np.empty((data.shape[0] + 31) // 32, np.uint32)
                    tickets.append((kind, late, srv.submit_lookup(key, data, out)))

        th = threading.Thread(target=submitter)
        th.start()
        lat = {"build": [], "lookup": []}
        failed = 0
        for got in range(len(trace)):
            while got >= len(tickets):
                time.sleep(0.0001)
            kind, late, t = tickets[got]
            try:
                ms, _ = srv.wait(t, packed=True)
            except cp.CpvsError:
                failed += 1  # e.g. a lookup whose DAG was evicted: the client would rebuild
                continue
            lat[kind].append(late + ms)
        wall = time.perf_counter() - t0
        th.join()
        stats = srv.stats()
        stats["requests_failed"] = failed
        srv.close()
        return lat, wall, stats

    def summ(lat, wall):
        allv = lat["build"] + lat["lookup"]
        r = lambda v: round(float(v), 3)  # noqa: E731
        return {"p50_ms": r(np.percentile(allv, 50)), "p99_ms": r(np.percentile(allv, 99)),
                "lookup_p50_ms": r(np.percentile(lat["lookup"], 50)), "lookup_p99_ms": r(np.percentile(lat["lookup"], 99)),
                "build_p50_ms": r(np.percentile(lat["build"], 50)), "build_p99_ms": r(np.percentile(lat["build"], 99)),
                "throughput_req_s": round(len(allv) / wall, 1), "wall_s": r(wall)}

    # warm both paths (plans, tuned lookups), then their capacities: the
    # same back-to-back trace (every request already due at t=0)
    burst = make_trace(1e9)[:600]
    plain_run(burst[:100])
    served_run(burst[:100])
    _, busy_plain = plain_run(burst)
    _, busy_served, _ = served_run(burst)
    cap_plain, cap_served = len(burst) / busy_plain, len(burst) / busy_served
    loads = {}
    for load in (0.8, 1.5):
        rate = load * cap_plain
        trace = make_trace(rate)
        lat_p, wall_p = plain_run(trace)
        lat_s, wall_s, stats = served_run(trace)
        loads[str(load)] = {"offered_req_s": round(rate, 1), "served": summ(lat_s, wall_s),
                            "plain_serial": summ(lat_p, wall_p),
                            "server_stats": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in stats.items()}}
    # under a budget that holds a few DAGs: evictions and admission by bytes
    budget = 12 << 20
    trace = make_trace(0.8 * cap_plain, recent=6)
    lat_p, wall_p = plain_run(trace)
    lat_s, wall_s, stats = served_run(trace, budget)
    budgeted = {"budget_bytes": budget, "offered_req_s": round(0.8 * cap_plain, 1),
                "lookups_target": "one of the 6 most recent builds",
                "served": summ(lat_s, wall_s), "plain_serial": summ(lat_p, wall_p),
                "server_stats": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in stats.items()}}
    head = loads["0.8"]
    return {"metric": "served p99 latency ms (c4)", "value": head["served"]["p99_ms"], "unit": "ms", "n_gpus": 1,
            "steps": nreq, "warmup": 100, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic: seeded scenes and Poisson request traces (no dataset)",
            "config": {"workload": "c4: " + WORKLOADS["c4"]["desc"], "requests_per_trace": nreq},
            "capacity_req_s": {"served": round(cap_served, 1), "plain_serial": round(cap_plain, 1)},
            "loads": loads, "budget_limited": budgeted}


def run_served(args):
    print(json.dumps(measure_served()), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--config", choices=tuple(WORKLOADS), default="c1")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="c1 line without the batched (c3), grid (c2) and served (c4) measurements")
    ap.add_argument("--part", choices=("all", "build", "lookup", "frame", "grid", "multi", "serve", "raster", "batch"),
                    default="all",
                    help="profiling aid: run one part alone (no contract line); see profile_part")
    ap.add_argument("--fixed-shapes", action="store_true",
                    help="profiling aid: default build launch shapes, no tuning replays")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        ap.error("--warmup must be at least 3")
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.config in ("c2", "c3"):
        run_batched(args)
    elif args.config == "c4":
        run_served(args)
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
