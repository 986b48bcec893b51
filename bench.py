#!/usr/bin/env python
"""Benchmark of the BVH hot path; headline = the 8M-triangle architectural scene.

Workload of one "step" (the headline): build_cwbvh_from_tris on 8,000,000
triangles of the architectural scene (40% from 200 tessellated axis-aligned
quads, 60% small clutter in a 20x6x20 box) with PLOC radius 14, distance 1 for
the first 3 passes, U64 Morton keys, no pre-splits or reinsertion, CWBVH8 with
at most 3 primitives per leaf (the medium_build PLOC settings of
src/lib.rs:270-281 through src/cwbvh/builder.rs:20-85).

  value        build throughput, Mtris/s, triangles already in HBM
  e2e          the same build through the public API from pinned host
               triangles: host->device copy and the CWBVH download included
  roofline     the headline build's dominant kernel against the measured HBM
               peak (algorithmic bytes per launch / event-timed launch time)
  cpu_baseline the C++ restatement of the reference (oracle) building the same
               8M scene on all host cores, and on 1 thread
  c3_*         16M incoherent closest-hit rays and 16M shadow rays on that tree
  c2_*         the 1M-triangle clustered scene with slow_build (pre-splits,
               radius 24, reinsertion 0.2, U128): build, e2e, 1920x1080
               primary rays and one cosine bounce per hit
  c1_*         10k triangles, PLOC radius 16 (build_ploc::<16>), 256x256 rays
  c4_*         512 scenes of 1k-200k triangles: one segmented build + one
               multi-BVH traversal vs a build and a traversal call per scene
  c5_*         the serving loop vs one request per call (Poisson 2,000/s)

--impl reference runs the CPU restatement of the reference's algorithm (the
Rust crate itself cannot be built on these machines) on the headline workload.
Multi-GPU: every rank builds its own replica (the path does not shard).
--detail PATH writes every measured figure to a JSON file as well.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PLOC build Mtris/s; CWBVH Mrays/s closest-hit; served p50/p99 latency"
WORKLOAD = "architectural-8M: PLOC r14 (distance 1 for 3 passes), U64 -> CWBVH8"
N_TRIS = 8_000_000
N_RAYS = 16_000_000
L2_FLUSH_BYTES = 512 << 20


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--tris", type=int, default=N_TRIS, help="headline scene size")
    ap.add_argument("--rays", type=int, default=N_RAYS, help="headline ray batch size (each kind)")
    ap.add_argument("--only", default="all", choices=["all", "c3", "c3-build", "c2", "c2-build", "c1", "c4", "c5"],
                    help="run one workload only (profiling); the JSON line then carries that workload")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving comparison (config 5)")
    ap.add_argument("--no-batched", action="store_true", help="skip the 512-scene batched comparison (config 4)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--detail", default="", help="also write every figure to this JSON file")
    return ap.parse_args(argv)


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def max_over_ranks(values, dist=None, device="cpu"):
    """Each value's maximum over the ranks (the slowest replica's time); the
    values themselves with one process."""
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def replica_rate(units, ms, world):
    """Whole-job throughput of `world` replicas that each process `units` in
    `ms` milliseconds (the slowest rank's time), in millions per second."""
    return world * units / (ms * 1e-3) / 1e6 if ms > 0 else 0.0


def r4(x):
    """Four significant digits (keeps the JSON line short)."""
    if x is None or isinstance(x, (bool, int, str)):
        return x
    return float(f"{x:.4g}")


class ClockSampler:
    """nvidia-smi sampling during the timed region (clocks and throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            # nvidia-smi takes a moment to start: wait for its first sample so
            # the timed region is covered
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < 3.0 and os.path.getsize(self.path) == 0:
                time.sleep(0.02)
        except Exception:
            self.proc = None
        return self

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_record(workload_key, kernel):
    """DRAM bytes per launch of `kernel` from an earlier ncu capture
    (profiles/traffic.json: workload -> kernel -> {bytes, commit, ...}), or
    None.  The figure is not measured by this run."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    rec = json.load(open(path)).get(workload_key, {}).get(kernel)
    return rec if isinstance(rec, dict) else None


ROOFLINE_NOTES = {
    "k_rs_pass": "radix sort passes: each pass is one wave of tiles whose ranking, look-back and scatter "
                 "phases are latency-bound",
    "k_resolve": "dependent rounds and tree climbs; bytes are a lower bound",
    "k_find": "branch-and-bound tree searches: each step a dependent node load",
    "k_ploc_coop": "nearest-neighbour search compute; clusters stay in L2",
    "k_ploc_cluster": "the last passes in shared memory: cluster barriers and the search's latency",
    "k_costs": "bottom-up climb: one dependent hand-off per level",
    "k_emit_all": "work queue over the tree: a node waits for its parent",
}


def reinsertion_schedule(n_nodes, ratio=0.2):
    """(candidates, searched) per reinsertion pass, as the reference's
    optimize_impl sizes them (src/bvh2/reinsertion.rs:101-115)."""
    out = []
    if ratio <= 0:
        return out
    for k in range(16):
        batch = max(int(np.float32(np.float32(n_nodes) * np.float32(ratio)) * np.float32(1.0 / (2 * k + 1))), 1)
        node_count = min(n_nodes, batch + 1)
        take = min(node_count * 2, n_nodes)
        out.append((take - 1, node_count - 1))
    return out


#: cost-record bytes per BVH2 node written by the cost pass and read by the
#: emission: the reference's 7 decisions of 8 bytes
#: (src/cwbvh/bvh2_to_cwbvh.rs:479-484), whatever record the kernels use
DEC_BYTES = 56


def kernel_byte_models(m, sum_counts, n_cw, n_prims, search_nodes=None, ratio=0.2, precision=1):
    """Algorithmic bytes of one build, per kernel (totals over its launches).

    Minimum bytes each kernel must move for its result, from the per-unit
    figures of the path's byte model.  The reinsertion searches read the node
    records the oracle counts for the same build (`search_nodes`, the same
    searches on the same tree); the other pointer-chasing kernels (k_resolve,
    k_costs, k_emit_all) also read tree nodes along their walks, which is not
    counted (a lower bound).  `precision` 1 = U128 Morton keys (the high 64
    bits sorted: 8 passes of 8 B keys), 0 = U64 (bits 24-63: 5 passes)."""
    nodes = 2 * m - 1
    sched = reinsertion_schedule(nodes, ratio)
    cand_sort = sum(4 * c * 16 for c, _ in sched) + sum(c * 4 for c, _ in sched)
    searched = sum(s_ for _, s_ in sched)
    sort_passes = 8 if precision else 5
    out = {
        # Morton sort on the high digits (key 8 B + value 4 B, read and
        # written per pass) and the reinsertion candidate sorts (u32 key + value)
        "k_rs_pass": sort_passes * m * 24 + cand_sort,
        # every PLOC pass: box read twice, offset byte written and read twice,
        # compacted cluster written; every merged pair written once
        "k_ploc_coop": sum_counts * (32 + 32 + 1 + 2 + 32) + (nodes - 1) * 32,
        # the last passes in shared memory: the clusters read once, the merged
        # pairs of those passes written
        "k_ploc_cluster": min(m, 32768) * 32 + 2 * min(m, 32768) * 32,
        # node + parent read, cost record written, children's records read
        "k_costs": nodes * (32 + 4 + DEC_BYTES) + (m - 1) * 2 * DEC_BYTES,
        # 80 B node and primitive indices written, each BVH2 node and record read
        "k_emit_all": n_cw * 80 + n_prims * 4 + nodes * (32 + DEC_BYTES),
        ("k_morton128" if precision else "k_morton64"): m * (32 + (16 if precision else 8) + 4),
        # leaves gathered into Morton order (U64: with the run fix-up, which
        # also reads the sorted code)
        ("k_gather" if precision else "k_fix_gather"): m * (4 + 32 + 32 + (0 if precision else 8)),
        "k_leaves_from_tris": m * (36 + 32),
        "k_reorder_tris": n_prims * (4 + 36 + 64),
    }
    if searched:
        # candidate id and result per search, 32 B per node record read
        out["k_find"] = searched * (4 + 16) + (search_nodes if search_nodes is not None else searched * 3) * 32
        # proposal read, conflict set written and read back
        out["k_resolve"] = sum(s_ * (16 + 32 + 32) for _, s_ in sched)
    return out


def build_byte_model(m, n_tris, sum_counts, n_cw, n_prims, ratio=0.2, precision=1):
    """Whole-build algorithmic bytes: triangle read, AABB write and read, Morton
    key + value, sort passes, PLOC, reinsertion sorts and proposals, CWBVH
    costs and nodes (the per-primitive byte model of the path)."""
    k = kernel_byte_models(m, sum_counts, n_cw, n_prims, ratio=ratio, precision=precision)
    return n_tris * 36 + m * (24 + 24) + sum(k.values())


def dominant_kernel(kernel_profile, models):
    """The build kernel with the largest share of event-timed device time that
    has a byte model: (name, launches, total_ms, share)."""
    build_kernels = {}
    for k, v in kernel_profile.items():
        if k.startswith("k_traverse"):
            continue
        k = "k_find" if k.startswith("k_find") else k  # one search kernel, two launch forms
        a = build_kernels.setdefault(k, {"launches": 0, "total_ms": 0.0})
        a["launches"] += v["launches"]
        a["total_ms"] += v["total_ms"]
    total = sum(v["total_ms"] for v in build_kernels.values())
    ranked = sorted(build_kernels.items(), key=lambda kv: -kv[1]["total_ms"])
    name, d = next(((k, v) for k, v in ranked if models.get(k)), ranked[0])
    return name, d["launches"], d["total_ms"], (d["total_ms"] / total if total else None)


class Bench:
    """Shared state of one GPU arm run: context, its stream, the L2 flush."""

    def __init__(self, args):
        import torch

        self.args = args
        self.rank, self.local_rank, self.world = dist_info()
        torch.cuda.set_device(self.local_rank)
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group("nccl", device_id=torch.device("cuda", self.local_rank))
            self.dist = dist
        import obvhs_gb300 as G

        self.G = G
        self.torch = torch
        self.ctx = G.Context(self.local_rank)
        self.stream = torch.cuda.ExternalStream(self.ctx.stream, device=torch.device("cuda", self.local_rank))
        self.flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def barrier(self):
        self.torch.cuda.synchronize()
        if self.dist:
            self.dist.barrier()

    def timed(self, fn, steps):
        """Runs fn() `steps` times; each call is bracketed by CUDA events on the
        library's stream and followed (outside the timing) by an L2 flush."""
        torch = self.torch
        ms = []
        for _ in range(steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(self.stream)
            fn()
            e1.record(self.stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            self.flush.fill_(1.0)
            torch.cuda.synchronize()
        return ms

    def trace_fn(self, cw, rays, out, kind):
        import ctypes

        lib, ctx = self.ctx.lib, self.ctx
        fn = {"closest": lib.obvhs_ray_traverse, "miss": lib.obvhs_ray_traverse_miss,
              "closest_ctri": lib.obvhs_ray_traverse_compressed}[kind]

        def run():
            ctx.check(fn(ctx.h, cw.h, ctypes.c_void_p(rays.data_ptr()), rays.shape[0],
                         ctypes.c_void_p(out.data_ptr()), 1))
        return run

    def e2e(self, tris_np, params, n_nodes, n_prims, steps, warmup):
        """The build through the public API from pinned host triangles, the
        CWBVH nodes and primitive indices downloaded into pinned host buffers;
        wall clock per step with the device idle on both sides."""
        import ctypes

        torch = self.torch
        h_tris = torch.from_numpy(tris_np).pin_memory().numpy()
        h_nodes = torch.empty((n_nodes, 80), dtype=torch.uint8).pin_memory().numpy()
        h_prims = torch.empty((n_prims,), dtype=torch.int32).pin_memory().numpy().view(np.uint32)
        ms = []
        self.e2e_steps_ms = []
        for i in range(warmup + steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b = self.G.build_cwbvh_from_tris(h_tris, params, ctx=self.ctx)
            self.ctx.check(self.ctx.lib.obvhs_cwbvh_download(self.ctx.h, b.h, h_nodes.ctypes.data_as(ctypes.c_void_p),
                                                             h_prims.ctypes.data_as(ctypes.c_void_p)))
            dt = (time.perf_counter() - t0) * 1e3
            if i >= warmup:
                ms.append(dt)
                self.e2e_steps_ms.append(round(dt, 3))
            self.flush.fill_(1.0)
            torch.cuda.synchronize()
            del b
        return sum(ms) / len(ms), len(tris_np) * 36, n_nodes * 80 + n_prims * 4

    def profile_build(self, d_tris, params):
        """Per-kernel device time of one build (events around every launch on
        the library's stream; not part of the timings)."""
        self.ctx.set_profiling(True)
        b = self.G.build_cwbvh_from_tris(d_tris, params, ctx=self.ctx)
        self.ctx.synchronize()
        prof = self.ctx.profile_report()
        self.ctx.set_profiling(False)
        del b
        return prof


def trav_forms(B: Bench, fn, n_rays, steps=3):
    """Mrays/s of a traversal call in every launch form of the context
    (block size x group stack in local (L) or shared (S) memory); the
    context is left in its default form."""
    out = {}
    try:
        for block, smem in B.G.Context.TRAVERSAL_CONFIGS:
            B.ctx.set_traversal_config(block, smem)
            fn()
            out[f"{block}{'S' if smem else 'L'}"] = r4(n_rays / (mean(B.timed(fn, steps)) * 1e-3) / 1e6)
    finally:
        B.ctx.set_traversal_config(0, False)
    return out


def config3(B: Bench, only_build=False):
    """The headline: the 8M architectural scene built PLOC -> CWBVH8, then 16M
    incoherent closest-hit and 16M shadow rays on the tree (device-resident)."""
    from obvhs_gb300 import scenes as S
    from obvhs_gb300.params import BvhBuildParams

    torch, G, args = B.torch, B.G, B.args
    p = BvhBuildParams(False, 14, 3, 0.0, 0.0, 0, 3, 3.0)
    tris = S.scene3_tris(args.tris)
    d_tris = torch.from_numpy(tris).cuda()
    holder = {}

    def build():
        holder["cw"] = G.build_cwbvh_from_tris(d_tris, p, ctx=B.ctx)

    for _ in range(args.warmup):
        build()
    B.barrier()
    clocks = ClockSampler(B.local_rank).start() if B.rank == 0 else None
    l0 = B.ctx.kernel_launches
    t_wall0 = time.perf_counter()
    build_ms = B.timed(build, args.steps)
    B.barrier()
    t_wall = time.perf_counter() - t_wall0
    launches = (B.ctx.kernel_launches - l0) // max(args.steps, 1)
    cw = holder["cw"]
    stats = cw.stats
    n_nodes, n_prims, _ = cw.info()
    out = {"tris": tris, "params": p, "build_ms": build_ms, "launches": launches, "stats": stats,
           "n_nodes": n_nodes, "n_prims": n_prims, "wall_s": t_wall, "clocks": None}
    if only_build:
        out["clocks"] = clocks.stop() if clocks else None
        return out

    closest, shadow = S.scene3_rays(args.rays)
    dc, ds = torch.from_numpy(closest).cuda(), torch.from_numpy(shadow).cuda()
    hits = torch.empty((len(closest), 2), dtype=torch.int32, device="cuda")
    miss = torch.empty((len(shadow),), dtype=torch.uint8, device="cuda")
    cw.set_triangles_compressed(d_tris)
    fc = B.trace_fn(cw, dc, hits, "closest")
    fs = B.trace_fn(cw, ds, miss, "miss")
    fcc = B.trace_fn(cw, dc, hits, "closest_ctri")
    for _ in range(args.warmup):
        fc(), fs(), fcc()
    B.barrier()
    tsteps = max(3, args.steps // 2)
    out["closest_ms"] = B.timed(fc, tsteps)
    out["shadow_ms"] = B.timed(fs, tsteps)
    out["closest_ctri_ms"] = B.timed(fcc, tsteps)
    out["clocks"] = clocks.stop() if clocks else None
    out["closest_by_form"] = trav_forms(B, fc, len(closest))
    fc()
    torch.cuda.synchronize()
    out["hit_fraction"] = float((hits[:, 0] != -1).float().mean().item())
    out["occluded_fraction"] = float((miss == 0).float().mean().item())
    out["n_closest"], out["n_shadow"] = len(closest), len(shadow)
    out["closest_sample"] = closest[:1_000_000]
    out["cw"] = cw
    del dc, ds
    out["profile"] = B.profile_build(d_tris, p)
    out["e2e_ms"], out["h2d"], out["d2h"] = B.e2e(tris, p, n_nodes, n_prims, args.steps, args.warmup)
    out["e2e_steps_ms"] = B.e2e_steps_ms
    return out


def config2(B: Bench, only_build=False):
    """The 1M clustered scene with slow_build; primary rays of a pinhole that
    frames the densest cluster, one cosine bounce per hit."""
    from obvhs_gb300 import scenes as S
    from obvhs_gb300.params import BvhBuildParams

    torch, G, args = B.torch, B.G, B.args
    p = BvhBuildParams.slow_build()
    tris, rays = S.scene2_tris(1_000_000), S.scene2_primary_rays()
    d_tris = torch.from_numpy(tris).cuda()
    holder = {}

    def build():
        holder["cw"] = G.build_cwbvh_from_tris(d_tris, p, ctx=B.ctx)

    for _ in range(args.warmup):
        build()
    B.barrier()
    l0 = B.ctx.kernel_launches
    build_ms = B.timed(build, args.steps)
    launches = (B.ctx.kernel_launches - l0) // max(args.steps, 1)
    cw = holder["cw"]
    stats = cw.stats
    n_nodes, n_prims, _ = cw.info()
    out = {"build_ms": build_ms, "launches": launches, "stats": stats, "n_nodes": n_nodes, "n_prims": n_prims}
    out["profile"] = B.profile_build(d_tris, p)
    if only_build:
        return out
    pid, pt = cw.ray_traverse(rays)
    bounce = S.bounce_rays(tris, rays, pid, pt)
    d_rays, d_bounce = torch.from_numpy(rays).cuda(), torch.from_numpy(bounce).cuda()
    out_p = torch.empty((len(rays), 2), dtype=torch.int32, device="cuda")
    out_b = torch.empty((max(len(bounce), 1), 2), dtype=torch.int32, device="cuda")
    fp = B.trace_fn(cw, d_rays, out_p, "closest")
    fb = B.trace_fn(cw, d_bounce, out_b, "closest")
    for _ in range(args.warmup):
        fp(), fb()
    B.barrier()
    out["primary_ms"] = B.timed(fp, args.steps)
    out["bounce_ms"] = B.timed(fb, args.steps)
    out["primary_by_form"] = trav_forms(B, fp, len(rays))
    out["bounce_by_form"] = trav_forms(B, fb, len(bounce))
    fb()
    torch.cuda.synchronize()
    out["n_primary"], out["n_bounce"] = len(rays), len(bounce)
    out["primary_hit_fraction"] = float((pid != 0xFFFFFFFF).mean())
    out["bounce_hit_fraction"] = float((out_b[:len(bounce), 0] != -1).float().mean().item())
    out["e2e_ms"], _, _ = B.e2e(tris, p, n_nodes, n_prims, args.steps, args.warmup)
    return out


def config1(B: Bench):
    """10k triangles, PLOC radius 16 (build_ploc::<16>, distance 1 never, U64)
    -> CWBVH (3 prims per leaf), 256x256 pinhole rays from (0,0,-3)."""
    from obvhs_gb300 import scenes as S
    from obvhs_gb300.params import BvhBuildParams

    torch, G, args = B.torch, B.G, B.args
    p = BvhBuildParams(False, 16, 0, 0.0, 0.0, 0, 3, 3.0)
    tris, rays = S.scene1()
    d_tris = torch.from_numpy(tris).cuda()
    holder = {}

    def build():
        holder["cw"] = G.build_cwbvh_from_tris(d_tris, p, ctx=B.ctx)

    for _ in range(args.warmup):
        build()
    build_ms = B.timed(build, args.steps)
    cw = holder["cw"]
    d_rays = torch.from_numpy(rays).cuda()
    hits = torch.empty((len(rays), 2), dtype=torch.int32, device="cuda")
    fc = B.trace_fn(cw, d_rays, hits, "closest")
    for _ in range(args.warmup):
        fc()
    ray_ms = B.timed(fc, args.steps)
    torch.cuda.synchronize()
    return {"build_ms": build_ms, "ray_ms": ray_ms, "n_tris": len(tris), "n_rays": len(rays),
            "hit_fraction": float((hits[:, 0] != -1).float().mean().item())}


def batched_scenes(G, ctx, base, n_scenes=512, seed=1004):
    """512 clustered scenes, triangle counts log-uniform over 1k-200k (scene i
    from the clustered generator with seed offset i), each with 4,096-262,144
    incoherent rays in proportion to its size.  The PLOC search radius, the
    traversal block size and stack depth come from the autotuner (a 64-scene
    sample).  Plain: every scene built and traced in its own calls.  Batched:
    one segmented build of all scenes, then one multi-BVH traversal launch.
    Device-resident inputs; wall clock with the device synchronised; hit ids
    and t compared between the two forms."""
    import torch
    from obvhs_gb300 import autotune as A
    from obvhs_gb300 import scenes as S
    from obvhs_gb300 import test_util as T

    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(1000), np.log(200_000), size=n_scenes)).astype(np.int64)
    tris, rays, owners = [], [], []
    for i, n in enumerate(sizes):
        t = S.scene2_tris(int(n), offset=i)
        tris.append(torch.from_numpy(t).cuda())
        k = int(4096 + (n - 1000) * (262_144 - 4096) / (200_000 - 1000))
        v = t.reshape(-1, 3)
        lo, hi = v.min(0), v.max(0)
        o = rng.uniform(lo, hi, size=(k, 3)).astype(np.float32)
        d = T.uniform_sample_sphere(rng.random(k).astype(np.float32), rng.random(k).astype(np.float32))
        rays.append(T.make_rays(o, d, 0.0, np.inf))
        owners.append(np.full(k, i, np.uint32))
    d_rays = [torch.from_numpy(r).cuda() for r in rays]
    all_rays = torch.from_numpy(np.concatenate(rays)).cuda()
    all_owner = torch.from_numpy(np.concatenate(owners).view(np.int32)).cuda()
    n_tris, n_rays = int(sizes.sum()), int(all_rays.shape[0])

    # autotune on a sample spread over the size range
    pick = A.sample_indices(sizes, 64)
    s_rays = torch.cat([d_rays[i] for i in pick])
    s_owner = torch.from_numpy(np.concatenate([np.full(len(rays[i]), j, np.int32) for j, i in enumerate(pick)])).cuda()
    p, tune = A.tune_segmented([tris[i] for i in pick], s_rays, s_owner, base, ctx=ctx)
    trav = tune["traversal"]
    ctx.set_traversal_config(trav["block"], trav["smem_stack"])

    def plain():
        out = []
        for t, r in zip(tris, d_rays):
            b = G.build_cwbvh_from_tris(t, p, ctx=ctx)
            out.append(b.ray_traverse(r))
            b.free()
        torch.cuda.synchronize()
        return out

    def batched():
        bvhs = G.build_cwbvh_from_tris_segmented(tris, p, ctx=ctx)
        hits = G.ray_traverse_multi(bvhs, all_owner, all_rays, ctx=ctx)
        torch.cuda.synchronize()
        return bvhs, hits

    try:
        plain()
        t0 = time.perf_counter()
        ref = plain()
        t_plain = time.perf_counter() - t0
        for b in batched()[0]:
            b.free()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bvhs, hits = batched()
        t_batched = time.perf_counter() - t0
        for b in bvhs:
            b.free()
        t0 = time.perf_counter()
        bvhs = G.build_cwbvh_from_tris_segmented(tris, p, ctx=ctx)
        torch.cuda.synchronize()
        t_build = time.perf_counter() - t0
        launches = bvhs[0].stats.kernel_launches if bvhs else 0
        t0 = time.perf_counter()
        hits = G.ray_traverse_multi(bvhs, all_owner, all_rays, ctx=ctx)
        torch.cuda.synchronize()
        t_trace = time.perf_counter() - t0
        for b in bvhs:
            b.free()
    finally:
        ctx.set_traversal_config(0, False)
    got = hits.cpu().numpy().view(np.uint32)
    exp = np.concatenate([np.stack([r.cpu().numpy().view(np.uint32)[:, 0], r.cpu().numpy().view(np.uint32)[:, 1]], 1)
                          for r in ref])
    identical = bool(np.array_equal(got, exp))
    return {"workload": f"{n_scenes} clustered scenes, 1k-200k triangles (log-uniform), "
                        "4,096-262,144 incoherent rays each", "preset": "medium_build",
            "tuned": {"radius": int(p.ploc_search_distance), "block": trav["block"],
                      "stack": "shared" if trav["smem_stack"] else "local"},
            "autotune": tune,
            "scenes": n_scenes, "triangles": n_tris, "rays": n_rays,
            "plain_s": t_plain, "batched_s": t_batched, "speedup": t_plain / t_batched,
            "batched_build_s": t_build, "batched_build_mtris_s": n_tris / t_build / 1e6,
            "batched_build_kernel_launches": launches,
            "batched_trace_mrays_s": n_rays / t_trace / 1e6, "identical_hits": identical}


def serving(params, n_requests=3000, rate=2000.0, budget=80 << 30, seed=1005):
    """The serving workload: Poisson arrivals (2,000 requests/s), 10% builds
    of 10k-2M clustered triangles that become resident BVHs, 90% ray batches
    of 1k-1M rays (log-uniform; half primary pinhole, half incoherent) against
    a resident BVH chosen by Zipf(1.1), LRU eviction under an 80 GB budget.
    Inputs are prefixes of 8 pooled 2M-triangle scenes and their 1M-ray
    batches in pinned host memory; 8 BVHs are resident before the first
    request.  The same stream runs through the continuous-batching server and
    the plain one-request-per-call server.  Every ray request brings its own
    pinned hit buffer (the client's), so hits are copied straight into it and
    a request is done when they have landed; after each run (outside the
    timing) the per-request hits are compared by a digest of the (id, t)
    words."""
    from obvhs_gb300 import serve as V

    tris, rays = V.clustered_pools(8, 2_000_000, 1_000_000, seed=seed)
    rng = np.random.default_rng(seed)
    reqs, scene_of = V.make_stream(n_requests, rate, tris, rays, rng, preloaded=8)
    pre = [(i, tris[scene_of[i]][:200_000]) for i in range(8)]
    ray_reqs = [r for r in reqs if r.kind == "rays"]
    hit_pool = V.pinned_empty((sum(len(r.rays) for r in ray_reqs), 2), np.uint32)
    at = 0
    for r in ray_reqs:
        r.out = hit_pool[at:at + len(r.rays)]
        at += len(r.rays)

    def digest(block):
        # (sum, xor) of the request's (id, t) words: any differing hit changes it
        w = block.view(np.uint64).ravel()
        return int(w.sum(dtype=np.uint64)), int(np.bitwise_xor.reduce(w)) if len(w) else 0

    be = V.GpuBackend(params)
    out = {}
    arrival = [r.arrival for r in reqs]

    def run(cls, squeeze):
        for r, a in zip(reqs, arrival):
            r.arrival, r.done, r.result, r.step = a * squeeze, None, None, -1
        hit_pool.fill(0xFFFFFFFF)
        srv = cls(be, budget)
        srv.run(reqs, preload=pre)
        return srv

    def release(srv):
        for k in list(srv.store.items):
            srv.store.items.pop(k)[0].free()

    try:
        # warm-up, untimed: the saturated stream once through each server, so
        # that the grow-only buffers (device scratch, pinned staging, output
        # pool) already have the sizes the largest steps need
        for cls in (V.ContinuousServer, V.PlainServer):
            release(run(cls, 0.05))
        results = {}
        # at the offered rate, then the same stream 20x compressed (40,000
        # requests/s: both servers saturated, throughput = capacity); three
        # runs per server in both, latency percentiles over all their
        # requests (one stall of the shared host does not set the tail) and
        # the median run's throughput (the saturated runs' throughput varies
        # by about +-10 % from run to run)
        for scen, squeeze, runs in (("", 1.0, 3), ("saturated_", 0.05, 3)):
            for name, cls in (("continuous", V.ContinuousServer), ("plain", V.PlainServer)):
                earlier, rates = [], []
                for _ in range(runs - 1):
                    srv = run(cls, squeeze)
                    earlier.append(V.snapshot(reqs))
                    rates.append(V.summarize(reqs)["mrays_s"])
                    release(srv)
                srv = run(cls, squeeze)
                summ = V.summarize(reqs, earlier)
                rates.append(summ["mrays_s"])
                summ["mrays_s_runs"] = rates
                summ["mrays_s"] = float(np.median(rates))
                summ["evictions"] = srv.store.evictions
                summ["rebuilds"] = srv.rebuilds
                if name == "continuous":
                    summ["launch_steps_build"] = srv.steps["build"]
                    summ["launch_steps_rays"] = srv.steps["rays"]
                out[scen + name] = summ
                results[scen + name] = [digest(r.out) if r.kind == "rays" else r.result for r in reqs]
                release(srv)
        out["identical_hits"] = (results["continuous"] == results["plain"] == results["saturated_continuous"]
                                 == results["saturated_plain"])
    finally:
        be.close()
    c, pl = out["continuous"], out["plain"]
    sc, sp = out["saturated_continuous"], out["saturated_plain"]
    out.update({"workload": f"{n_requests} requests, Poisson {rate:.0f}/s, 10% builds (10k-2M tris) / 90% ray "
                            "batches (1k-1M rays, half primary, half incoherent), Zipf(1.1) targets, "
                            f"{budget >> 30} GB budget, LRU", "preset": "medium_build",
                "p99_speedup_rays": pl["latency_rays"]["p99_ms"] / c["latency_rays"]["p99_ms"],
                "throughput_ratio_offered": c["mrays_s"] / pl["mrays_s"],
                "capacity_ratio": sc["mrays_s"] / sp["mrays_s"],
                "capacity_mrays_s": sc["mrays_s"], "capacity_mrays_s_plain": sp["mrays_s"]})
    return out


def oracle_build_s(tris, params, nthreads, reps=1):
    """Seconds per oracle build of the whole scene on `nthreads` host threads."""
    from oracle import oracle as O

    t = []
    ob = None
    for _ in range(reps):
        t0 = time.perf_counter()
        ob = O.build(tris=tris, params=params, nthreads=nthreads, keep_intermediate=False)
        t.append(time.perf_counter() - t0)
    return t, ob


def cpu_baseline(c3, cores):
    """The oracle on the headline scene: one full build on all host threads,
    one on a single thread, and a 1M-ray sample of the closest-hit rays traced
    on the GPU-built tree with node-visit / triangle-test counters (which also
    give the traversal's algorithmic bytes)."""
    from oracle import oracle as O

    tris, p = c3["tris"], c3["params"]
    t_all, _ = oracle_build_s(tris, p, cores)
    t_one, _ = oracle_build_s(tris, p, 1)
    nodes, pidx = c3["cw"].download()
    sample = c3["closest_sample"]
    t0 = time.perf_counter()
    _, _, _, cnt = O.traverse(nodes, pidx, tris, sample, 0, nthreads=cores, counters=True)
    dt = time.perf_counter() - t0
    n = len(tris)
    return {"value": n / t_all[0] / 1e6, "value_1thread": n / t_one[0] / 1e6, "s_all": t_all[0], "s_1": t_one[0],
            "mrays_s": len(sample) / dt / 1e6, "visits_per_ray": cnt[0] / len(sample),
            "tests_per_ray": cnt[1] / len(sample)}


def run_reference(args):
    rank, _, world = dist_info()
    if rank != 0:
        return
    from obvhs_gb300 import scenes as S
    from obvhs_gb300.params import BvhBuildParams

    tris = S.scene3_tris(args.tris)
    cores = os.cpu_count() or 1
    p = BvhBuildParams(False, 14, 3, 0.0, 0.0, 0, 3, 3.0)
    oracle_build_s(tris, p, cores, args.warmup)
    times, _ = oracle_build_s(tris, p, cores, args.steps)
    ms = 1e3 * sum(times) / len(times)
    rate = len(tris) / (ms * 1e-3) / 1e6
    sample = f"full {len(tris)}-triangle build per step, {cores} threads"
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "Mtris/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded PCG64)",
        "config": {"workload": WORKLOAD, "n_tris": len(tris),
                   "implementation": "C++ restatement of obvhs 0.3.1 (oracle/); the Rust crate cannot be built here"},
        "cpu_baseline": {"value": rate, "unit": "Mtris/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": "Mtris/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def mean(x):
    return sum(x) / len(x) if x else 0.0


def run_gb300(args):
    B = Bench(args)
    world = B.world
    only = args.only
    detail = {}

    if only in ("c2", "c2-build"):
        c2 = config2(B, only_build=only == "c2-build")
        if B.rank == 0:
            m = mean(c2["build_ms"])
            print(json.dumps({"metric": METRIC, "value": replica_rate(1_000_000, m, world), "unit": "Mtris/s",
                              "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": m,
                              "config": {"workload": "clustered-1M-slow_build"}}), flush=True)
        return
    if only in ("c4", "c5"):
        from obvhs_gb300.params import BvhBuildParams

        res = (batched_scenes(B.G, B.ctx, BvhBuildParams.medium_build()) if only == "c4"
               else serving(BvhBuildParams.medium_build()))
        if B.rank == 0:
            keep = {k: v for k, v in res.items() if not isinstance(v, dict) or k in ("tuned", "autotune")}
            for k in ("continuous", "plain", "saturated_continuous", "saturated_plain"):
                if k in res:
                    keep[k] = {"mrays_s": r4(res[k]["mrays_s"]),
                               "rays_p50_p99_ms": [r4(res[k]["latency_rays"]["p50_ms"]),
                                                   r4(res[k]["latency_rays"]["p99_ms"])],
                               "builds_p99_ms": r4(res[k]["latency_builds"]["p99_ms"])}
            print(json.dumps({"metric": METRIC, "config": {"workload": only}, **keep}, default=str), flush=True)
        return
    if only == "c1":
        c1 = config1(B)
        if B.rank == 0:
            m = mean(c1["build_ms"])
            print(json.dumps({"metric": METRIC, "value": c1["n_tris"] / (m * 1e-3) / 1e6, "unit": "Mtris/s",
                              "ms_per_step": m, "rays_mrays_s": c1["n_rays"] / (mean(c1["ray_ms"]) * 1e-3) / 1e6,
                              "config": {"workload": "uniform-10k r16"}}), flush=True)
        return

    c3 = config3(B, only_build=only == "c3-build")
    n = len(c3["tris"])
    m_build = mean(c3["build_ms"])
    if only == "c3-build":
        m_build, = max_over_ranks([m_build], B.dist, "cuda")
        if B.rank == 0:
            print(json.dumps({"metric": METRIC, "value": replica_rate(n, m_build, world), "unit": "Mtris/s",
                              "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": m_build,
                              "gpu_launches": c3["launches"], "config": {"workload": WORKLOAD, "n_tris": n}}),
                  flush=True)
        return
    m_e2e, m_cl, m_sh = mean([c3["e2e_ms"]]), mean(c3["closest_ms"]), mean(c3["shadow_ms"])
    m_build, m_e2e, m_cl, m_sh = max_over_ranks([m_build, m_e2e, m_cl, m_sh], B.dist, "cuda")
    if B.rank != 0:
        if B.dist:
            B.dist.destroy_process_group()
        return
    value = replica_rate(n, m_build, world)
    e2e = replica_rate(n, m_e2e, world)

    c2 = config2(B) if only == "all" else None
    c1 = config1(B) if only == "all" else None
    from obvhs_gb300.params import BvhBuildParams

    batch = None if (args.no_batched or only != "all") else batched_scenes(B.G, B.ctx, BvhBuildParams.medium_build())
    served = None if (args.no_serving or only != "all") else serving(BvhBuildParams.medium_build())
    cores = os.cpu_count() or 1
    cpu = None if args.no_cpu else cpu_baseline(c3, cores)

    # roofline of the headline build's dominant kernel (largest share of
    # event-timed device time in one profiled build): algorithmic bytes per
    # launch / mean launch time
    peak, peak_kind = measured_peak()
    st = c3["stats"]
    models = kernel_byte_models(st.leaf_count, st.ploc_sum_counts, c3["n_nodes"], c3["n_prims"], ratio=0.0,
                                precision=0)
    dom, dom_launches, dom_total, dom_share = dominant_kernel(c3["profile"], models)
    dom_launches = max(dom_launches, 1)
    dom_bytes = models.get(dom, 0) / dom_launches
    dom_ms = dom_total / dom_launches
    dom_achieved = dom_bytes / (dom_ms * 1e-3) / 1e9 if dom_ms > 0 else 0.0
    traffic = traffic_record("architectural-8M", dom)
    build_bytes = build_byte_model(st.leaf_count, n, st.ploc_sum_counts, c3["n_nodes"], c3["n_prims"], ratio=0.0,
                                   precision=0)
    build_achieved = build_bytes / (m_build * 1e-3) / 1e9

    line = {
        "metric": METRIC, "value": r4(value), "unit": "Mtris/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r4(m_build), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded PCG64 scenes)",
        "config": {"workload": WORKLOAD, "n_tris": n, "cwbvh_nodes": c3["n_nodes"],
                   "l2": "inputs 288 MB > L2, and a 512 MB flush between timed steps",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": r4(e2e), "unit": "Mtris/s", "h2d_bytes_per_step": c3["h2d"], "d2h_bytes_per_step": c3["d2h"],
                "ms_per_step": r4(m_e2e)},
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": r4(dom_achieved), "peak": peak,
                     "unit": "GB/s", "frac": r4(dom_achieved / peak), "peak_kind": peak_kind,
                     "traffic": traffic["bytes"] if traffic else None,
                     "traffic_src": (f"ncu capture at commit {traffic['commit']} (profiles/traffic.json), "
                                     "not this run") if traffic else None,
                     "alg_bytes_per_launch": r4(dom_bytes), "launches": dom_launches, "mean_launch_ms": r4(dom_ms),
                     "share": r4(dom_share)},
        "roofline_build": {"achieved": r4(build_achieved), "frac": r4(build_achieved / peak),
                           "bytes_per_tri": r4(build_bytes / n)},
        "gpu_launches": c3["launches"],
        "clocks": c3["clocks"],
        "c3_closest_mrays_s": r4(replica_rate(c3["n_closest"], m_cl, world)),
        "c3_shadow_mrays_s": r4(replica_rate(c3["n_shadow"], m_sh, world)),
        "c3_closest_ctri_mrays_s": r4(replica_rate(c3["n_closest"], mean(c3["closest_ctri_ms"]), world)),
        "c3_hit_frac": r4(c3["hit_fraction"]),
        "c3_closest_by_form": c3["closest_by_form"],
    }
    if cpu:
        line["cpu_baseline"] = {"value": r4(cpu["value"]), "unit": "Mtris/s", "cores": cores, "kind": "port",
                                "sample": f"1 full {n}-tri build per thread count ({cpu['s_all']:.1f} s, "
                                          f"{cpu['s_1']:.1f} s)",
                                "value_1thread": r4(cpu["value_1thread"]), "c3_closest_mrays_s": r4(cpu["mrays_s"])}
        alg = 40.0 + 80.0 * cpu["visits_per_ray"] + 36.0 * cpu["tests_per_ray"]
        ach = alg * c3["n_closest"] / (m_cl * 1e-3) / 1e9
        line["roofline_c3_closest"] = {"achieved": r4(ach), "frac": r4(ach / peak), "bytes_per_ray": r4(alg)}
    if c2:
        s2 = c2["stats"]
        line.update({
            "c2_build_mtris_s": r4(1.0 / (mean(c2["build_ms"]) * 1e-3)),
            "c2_e2e_mtris_s": r4(1.0 / (c2["e2e_ms"] * 1e-3)),
            "c2_stages_ms": [r4(x) for x in s2.stage_ms],
            "c2_primary_mrays_s": r4(c2["n_primary"] / (mean(c2["primary_ms"]) * 1e-3) / 1e6),
            "c2_bounce_mrays_s": r4(c2["n_bounce"] / (mean(c2["bounce_ms"]) * 1e-3) / 1e6),
            "c2_primary_hit_frac": r4(c2["primary_hit_fraction"]), "c2_bounce_rays": c2["n_bounce"],
            "c2_launches": c2["launches"],
            "c2_bounce_by_form": c2["bounce_by_form"],
        })
    if c1:
        line.update({"c1_build_mtris_s": r4(c1["n_tris"] / (mean(c1["build_ms"]) * 1e-3) / 1e6),
                     "c1_build_ms": r4(mean(c1["build_ms"])),
                     "c1_mrays_s": r4(c1["n_rays"] / (mean(c1["ray_ms"]) * 1e-3) / 1e6)})
    if batch:
        line.update({"c4_speedup": r4(batch["speedup"]), "c4_build_mtris_s": r4(batch["batched_build_mtris_s"]),
                     "c4_trace_mrays_s": r4(batch["batched_trace_mrays_s"]), "c4_tuned": batch["tuned"],
                     "c4_identical": batch["identical_hits"]})
    if served:
        c = served["continuous"]["latency_rays"]
        line.update({"c5_capacity_ratio": r4(served["capacity_ratio"]),
                     "c5_mrays_s": r4(served["capacity_mrays_s"]),
                     "c5_rays_p50_p99_p999_ms": [r4(c["p50_ms"]), r4(c["p99_ms"]), r4(c["p999_ms"])],
                     "c5_p99_speedup": r4(served["p99_speedup_rays"]), "c5_identical": served["identical_hits"]})
    if args.detail:
        detail.update({"line": line, "c3_profile": c3["profile"], "c3_build_ms": c3["build_ms"],
                       "c3_e2e_steps_ms": c3.get("e2e_steps_ms"),
                       "c3_stage_ms": list(st.stage_ms), "c3_wall_s": c3["wall_s"], "cpu": cpu,
                       "kernel_models": models})
        if c2:
            detail.update({"c2_primary_by_form": c2["primary_by_form"], "c2_profile": c2["profile"],
                           "c2_build_ms": c2["build_ms"],
                           "c2": {k: v for k, v in c2.items() if k not in ("stats", "profile")}})
        if c1:
            detail["c1"] = c1
        detail["batched"] = batch
        detail["serving"] = served
        with open(args.detail, "w") as f:
            json.dump(detail, f, indent=1, default=str)
    print(json.dumps(line), flush=True)
    if B.dist:
        B.dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
