#!/usr/bin/env python
"""Benchmark of the BVH hot path on the 1M-triangle clustered scene.

Workload (one "step"): build_cwbvh_from_tris on 1,000,000 triangles in 64
Gaussian clusters with the slow_build preset (pre-splits, PLOC radius 24 with
distance 1 for 2 passes, reinsertion ratio 0.2, U128 Morton keys, 3 primitives
per leaf), plus, timed separately, closest-hit traversal of the 1920x1080
primary rays and of one cosine-weighted bounce ray per primary hit.

  value       build throughput, Mtris/s, triangles already in HBM
  e2e         the same build through the public API from pinned host
              triangles, host->device copy and the CWBVH download included
  traversal   Mrays/s of the primary and bounce batches (device-resident rays)
  roofline    the build's dominant kernel against the measured HBM peak
              (also the whole build, and the primary traversal kernel)
  cpu_baseline the C++ restatement of the reference (oracle) on all host cores

--impl reference runs that CPU restatement of the reference's algorithm (the
Rust crate itself cannot be built on these machines) on the same workload.
Multi-GPU: every rank builds its own replica (the path does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PLOC build Mtris/s; CWBVH Mrays/s closest-hit; served p50/p99 latency"
WORKLOAD = "clustered-1M-slow_build"
N_TRIS = 1_000_000
L2_FLUSH_BYTES = 512 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--tris", type=int, default=N_TRIS)
    ap.add_argument("--no-serving", action="store_true",
                    help="skip the serving run (Poisson request stream, resident BVHs, continuous batching)")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the 512-scene batched build + traversal comparison")
    ap.add_argument("--no-arch-scene", action="store_true",
                    help="skip the 8M-triangle architectural scene (build + 16M incoherent + 16M shadow rays)")
    return ap.parse_args()


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


ROOFLINE_NOTES = {
    "k_rs_pass": "radix sort passes of 0.03-1M keys: each pass is one wave of tiles whose ranking, "
                 "decoupled look-back and scatter phases are latency-bound",
    "k_resolve": "dependent rounds and tree climbs; bytes are a lower bound",
    "k_find": "branch-and-bound tree searches: each step a dependent node load (bytes: the node records the "
              "oracle's searches read on the same tree)",
    "k_ploc_coop": "compute in the nearest-neighbour search; clusters stay in L2",
    "k_ploc_cluster": "the last passes in shared memory: cluster barriers and the search's latency",
    "k_costs": "bottom-up tree climb; bytes are a lower bound",
    "k_emit_all": "work queue over the tree; bytes are a lower bound",
}


def reinsertion_schedule(n_nodes, ratio=0.2):
    """(candidates, searched) per reinsertion pass, as the reference's
    optimize_impl sizes them (src/bvh2/reinsertion.rs:101-115)."""
    out = []
    for k in range(16):
        batch = max(int(np.float32(np.float32(n_nodes) * np.float32(ratio)) * np.float32(1.0 / (2 * k + 1))), 1)
        node_count = min(n_nodes, batch + 1)
        take = min(node_count * 2, n_nodes)
        out.append((take - 1, node_count - 1))
    return out


def kernel_byte_models(m, sum_counts, n_cw, n_prims, search_nodes=None):
    """Algorithmic bytes of one build, per kernel (totals over its launches).

    Minimum bytes each kernel must move for its result, from the per-unit
    figures of the path's byte model.  The reinsertion searches read the node
    records the oracle counts for the same build (`search_nodes`, the same
    searches on the same tree); the other pointer-chasing kernels (k_resolve,
    k_costs, k_emit_all) also read tree nodes along their walks, which is not
    counted (a lower bound)."""
    nodes = 2 * m - 1
    sched = reinsertion_schedule(nodes)
    cand_sort = sum(4 * c * 16 for c, _ in sched) + sum(c * 4 for c, _ in sched)
    searched = sum(s_ for _, s_ in sched)
    return {
        # Morton sort on the high 64 bits (8 passes of 8-bit digits over key
        # 8 B + value 4 B, read and written) and the 16 candidate sorts (u32
        # key + value)
        "k_rs_pass": 8 * m * 24 + cand_sort,
        # every PLOC pass: box read twice, offset byte written and read twice,
        # compacted cluster written; every merged pair written once
        "k_ploc_coop": sum_counts * (32 + 32 + 1 + 2 + 32) + (nodes - 1) * 32,
        # the last passes in shared memory: the clusters read once, the merged
        # pairs of those passes written
        "k_ploc_cluster": min(m, 32768) * 32 + 2 * min(m, 32768) * 32,
        # candidate id and result per search, 32 B per node record read
        "k_find": searched * (4 + 16) + (search_nodes if search_nodes is not None else searched * 3) * 32,
        # proposal read, conflict set written and read back
        "k_resolve": sum(s_ * (16 + 32 + 32) for _, s_ in sched),
        # node + parent read, cost record (96 B) written, children records read
        "k_costs": nodes * (32 + 4 + 96) + (m - 1) * 2 * 96,
        # 80 B node and primitive indices written, each BVH2 node and record read
        "k_emit_all": n_cw * 80 + n_prims * 4 + nodes * (32 + 96),
        "k_morton128": m * (32 + 16),
        "k_gather": m * (4 + 32 + 32),
        "k_leaves_from_tris": m * (36 + 32),
        "k_reorder_tris": n_prims * (4 + 36 + 64),
    }


def build_byte_model(m, n_tris, sum_counts, n_cw, n_prims):
    """Whole-build algorithmic bytes: triangle read, AABB write and read, Morton
    key + value, 16 sort passes, PLOC, reinsertion sorts and proposals, CWBVH
    costs and nodes (the per-primitive byte model of the path)."""
    k = kernel_byte_models(m, sum_counts, n_cw, n_prims)
    return n_tris * 36 + m * (24 + 24) + sum(k.values())


def arch_scene(ctx, stream, steps, warmup, flush):
    """The 8M-triangle architectural scene: PLOC (radius 14, distance 1 for 3
    passes, U64) -> CWBVH build, then 16M incoherent closest-hit rays and 16M
    shadow rays to 4 point lights, all device-resident, CUDA-event timed."""
    import ctypes
    import torch
    import obvhs_gb300 as G
    from obvhs_gb300 import scenes as S
    from obvhs_gb300.params import BvhBuildParams

    tris = S.scene3_tris(8_000_000)
    closest, shadow = S.scene3_rays(16_000_000)
    d = torch.from_numpy(tris).cuda()
    dc, ds = torch.from_numpy(closest).cuda(), torch.from_numpy(shadow).cuda()
    plain = BvhBuildParams(False, 14, 3, 0.0, 0.0, 0, 3, 3.0)

    def timed(fn, k):
        ms = []
        for _ in range(k):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            flush.fill_(1.0)
            torch.cuda.synchronize()
        return sum(ms) / len(ms)

    holder = {}

    def build(p):
        holder["cw"] = G.build_cwbvh_from_tris(d, p, ctx=ctx)

    for _ in range(warmup):
        build(plain)
    plain_ms = timed(lambda: build(plain), steps)
    medium = BvhBuildParams.medium_build()
    for _ in range(warmup):
        build(medium)
    medium_ms = timed(lambda: build(medium), steps)
    build(plain)
    cw = holder["cw"]
    out = torch.empty((len(closest), 2), dtype=torch.int32, device="cuda")
    miss = torch.empty((len(shadow),), dtype=torch.uint8, device="cuda")
    lib = ctx.lib

    def trace():
        ctx.check(lib.obvhs_ray_traverse(ctx.h, cw.h, ctypes.c_void_p(dc.data_ptr()), len(closest),
                                         ctypes.c_void_p(out.data_ptr()), 1))

    def occlude():
        ctx.check(lib.obvhs_ray_traverse_miss(ctx.h, cw.h, ctypes.c_void_p(ds.data_ptr()), len(shadow),
                                              ctypes.c_void_p(miss.data_ptr()), 1))

    def trace_ctri():
        ctx.check(lib.obvhs_ray_traverse_compressed(ctx.h, cw.h, ctypes.c_void_p(dc.data_ptr()), len(closest),
                                                    ctypes.c_void_p(out.data_ptr()), 1))

    cw.set_triangles_compressed(d)
    for _ in range(warmup):
        trace()
        occlude()
        trace_ctri()
    cc_ms = timed(trace_ctri, steps)
    c_ms = timed(trace, steps)
    s_ms = timed(occlude, steps)
    n = len(tris)
    return {"workload": "architectural-8M: 200 tessellated quads + clutter, 16M incoherent + 16M shadow rays",
            "n_tris": n, "build_plain_ms": plain_ms, "build_plain_mtris_s": n / (plain_ms * 1e-3) / 1e6,
            "build_plain": "PLOC radius 14, distance-1 for 3 passes, U64 -> CWBVH (3 prims/leaf)",
            "build_medium_build_ms": medium_ms, "build_medium_build_mtris_s": n / (medium_ms * 1e-3) / 1e6,
            "incoherent_closest_mrays_s": len(closest) / (c_ms * 1e-3) / 1e6, "incoherent_closest_ms": c_ms,
            "shadow_any_hit_mrays_s": len(shadow) / (s_ms * 1e-3) / 1e6, "shadow_any_hit_ms": s_ms,
            "incoherent_closest_compressed_tris_mrays_s": len(closest) / (cc_ms * 1e-3) / 1e6,
            "hit_fraction": float((out[:, 0] != -1).float().mean().item())}


def batched_scenes(G, ctx, base, n_scenes=512, seed=1004):
    """512 clustered scenes, triangle counts log-uniform over 1k-200k (scene i
    from the clustered generator with seed offset i), each with 4,096-262,144
    incoherent rays in proportion to its size.  The PLOC search radius comes
    from the autotuner (segmented build + multi-BVH traversal of a 64-scene
    sample, radius 8 / 14 / 24).  Plain: every scene built and traced in its
    own calls.  Batched: one segmented build of all scenes, then one multi-BVH
    traversal launch.  Device-resident inputs; wall clock with the device
    synchronised; hit ids and t compared between the two forms."""
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
    got = hits.cpu().numpy().view(np.uint32)
    exp = np.concatenate([np.stack([r.cpu().numpy().view(np.uint32)[:, 0], r.cpu().numpy().view(np.uint32)[:, 1]], 1)
                          for r in ref])
    identical = bool(np.array_equal(got, exp))
    return {"workload": f"{n_scenes} clustered scenes, 1k-200k triangles (log-uniform), "
                        "4,096-262,144 incoherent rays each", "preset": "medium_build",
            "search_radius": int(p.ploc_search_distance),
            "autotune_s_by_radius": {str(k): v for k, v in tune.items()},
            "scenes": n_scenes, "triangles": n_tris, "rays": n_rays,
            "plain_s": t_plain, "batched_s": t_batched, "speedup": t_plain / t_batched,
            "plain_scenes_per_s": n_scenes / t_plain, "batched_scenes_per_s": n_scenes / t_batched,
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
    try:
        # warm-up on a short stream of the same kind
        wreqs, wsc = V.make_stream(200, rate, tris, rays, np.random.default_rng(seed + 1), preloaded=8)
        V.ContinuousServer(be, budget).run(wreqs, preload=pre)
        V.PlainServer(be, budget).run(wreqs, preload=pre)
        results = {}
        arrival = [r.arrival for r in reqs]
        # at the offered rate, then the same stream 20x compressed (40,000
        # requests/s: both servers saturated, throughput = capacity)
        for scen, squeeze in (("", 1.0), ("saturated_", 0.05)):
            for name, cls in (("continuous", V.ContinuousServer), ("plain", V.PlainServer)):
                for r, a in zip(reqs, arrival):
                    r.arrival, r.done, r.result, r.step = a * squeeze, None, None, -1
                hit_pool.fill(0xFFFFFFFF)
                srv = cls(be, budget)
                srv.run(reqs, preload=pre)
                summ = V.summarize(reqs)
                summ["evictions"] = srv.store.evictions
                summ["rebuilds"] = srv.rebuilds
                if name == "continuous":
                    summ["launch_steps_build"] = srv.steps["build"]
                    summ["launch_steps_rays"] = srv.steps["rays"]
                out[scen + name] = summ
                results[scen + name] = [digest(r.out) if r.kind == "rays" else r.result for r in reqs]
                for k in list(srv.store.items):
                    srv.store.items.pop(k)[0].free()
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


def workload(n):
    from obvhs_gb300 import scenes as S

    return S.scene2_tris(n), S.scene2_primary_rays()


def cpu_build_rate(tris, params, reps, nthreads):
    """Oracle builds of the full scene on `nthreads` host threads: Mtris/s."""
    from oracle import oracle as O

    t = []
    for _ in range(reps):
        t0 = time.perf_counter()
        ob = O.build(tris=tris, params=params, nthreads=nthreads, keep_intermediate=False)
        t.append(time.perf_counter() - t0)
    cpu_build_rate.last = ob
    return len(tris) / (sum(t) / len(t)) / 1e6, t


def cpu_baseline(tris, params, rays, cores, ctx):
    """The oracle: two builds, and the primary rays traced on the GPU-built
    tree with visit/test counters (all host threads)."""
    from oracle import oracle as O

    rate, times = cpu_build_rate(tris, params, 2, cores)
    ob = cpu_build_rate.last
    import obvhs_gb300 as G

    cw = G.build_cwbvh_from_tris(tris, params, ctx=ctx)
    nodes, pidx = cw.download()
    t0 = time.perf_counter()
    _, _, _, cnt = O.traverse(nodes, pidx, tris, rays, 0, nthreads=cores, counters=True)
    dt = time.perf_counter() - t0
    return rate, times, {"visits": int(cnt[0]), "tests": int(cnt[1]), "mrays_s": len(rays) / dt / 1e6,
                         "searches": ob.searches, "search_nodes": ob.search_nodes}


def run_reference(args):
    rank, _, world = dist_info()
    if rank != 0:
        return
    from obvhs_gb300.params import BvhBuildParams

    tris, _ = workload(args.tris)
    cores = os.cpu_count() or 1
    p = BvhBuildParams.slow_build()
    for _ in range(args.warmup):
        cpu_build_rate(tris, p, 1, cores)
    rate, times = cpu_build_rate(tris, p, args.steps, cores)
    ms = 1e3 * sum(times) / len(times)
    sample = f"full {len(tris)}-triangle slow_build per step, {cores} threads"
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "Mtris/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded PCG64)",
        "config": {"workload": WORKLOAD, "n_tris": len(tris), "preset": "slow_build",
                   "implementation": "C++ restatement of obvhs 0.3.1 (oracle/); the Rust crate cannot be built here"},
        "cpu_baseline": {"value": rate, "unit": "Mtris/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": "Mtris/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gb300(args):
    import torch

    rank, local_rank, world = dist_info()
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    import obvhs_gb300 as G
    from obvhs_gb300 import scenes as S
    from obvhs_gb300.params import BvhBuildParams

    ctx = G.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local_rank))
    tris, rays = workload(args.tris)
    p = BvhBuildParams.slow_build()
    d_tris = torch.from_numpy(tris).cuda()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    # rays: primary, and bounce rays from the primary hits
    cw = G.build_cwbvh_from_tris(d_tris, p, ctx=ctx)
    pid, pt = cw.ray_traverse(rays)
    bounce = S.bounce_rays(tris, rays, pid, pt)
    d_rays = torch.from_numpy(rays).cuda()
    d_bounce = torch.from_numpy(bounce).cuda()
    n_nodes, n_prims, _ = cw.info()
    del cw

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    def timed(fn, steps):
        """Runs fn() `steps` times; each call is bracketed by CUDA events on the
        library's stream and followed (outside the timing) by an L2 flush."""
        ms = []
        for _ in range(steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            flush.fill_(1.0)
            torch.cuda.synchronize()
        return ms

    def build_once():
        b = G.build_cwbvh_from_tris(d_tris, p, ctx=ctx)
        build_once.last = b

    for _ in range(args.warmup):
        build_once()
    barrier()
    clocks = ClockSampler(local_rank).start() if rank == 0 else None
    l0 = ctx.kernel_launches
    t_wall0 = time.perf_counter()
    build_ms = timed(build_once, args.steps)
    barrier()
    t_wall = time.perf_counter() - t_wall0
    launches = (ctx.kernel_launches - l0) // max(args.steps, 1)
    stats = build_once.last.stats
    cw = build_once.last

    # traversal (device-resident rays), each step = primary + bounce batch
    out_p = torch.empty((len(rays), 2), dtype=torch.int32, device="cuda")
    out_b = torch.empty((max(len(bounce), 1), 2), dtype=torch.int32, device="cuda")
    lib = ctx.lib
    import ctypes

    def trace(r, out):
        ctx.check(lib.obvhs_ray_traverse(ctx.h, cw.h, ctypes.c_void_p(r.data_ptr()), r.shape[0],
                                         ctypes.c_void_p(out.data_ptr()), 1))

    for _ in range(args.warmup):
        trace(d_rays, out_p)
        trace(d_bounce, out_b)
    barrier()
    prim_ms = timed(lambda: trace(d_rays, out_p), args.steps)
    bounce_ms = timed(lambda: trace(d_bounce, out_b), args.steps) if len(bounce) else [0.0]
    clk = clocks.stop() if clocks else None

    # per-kernel device time of one build and one primary batch (events around
    # every launch on the library's stream; not part of the timings above)
    ctx.set_profiling(True)
    b = G.build_cwbvh_from_tris(d_tris, p, ctx=ctx)
    trace(d_rays, out_p)
    ctx.synchronize()
    kernel_profile = ctx.profile_report()
    ctx.set_profiling(False)
    del b

    # e2e through the public API: pinned host triangles in, CWBVH nodes out
    h_tris = torch.from_numpy(tris).pin_memory()
    h_nodes = torch.empty((n_nodes, 80), dtype=torch.uint8).pin_memory().numpy()
    h_prims = torch.empty((n_prims,), dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    h_tris_np = h_tris.numpy()
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b = G.build_cwbvh_from_tris(h_tris_np, p, ctx=ctx)
        ctx.check(lib.obvhs_cwbvh_download(ctx.h, b.h, h_nodes.ctypes.data_as(ctypes.c_void_p),
                                           h_prims.ctypes.data_as(ctypes.c_void_p)))
        dt = (time.perf_counter() - t0) * 1e3
        if i >= args.warmup:
            e2e_ms.append(dt)
        flush.fill_(1.0)
        torch.cuda.synchronize()
        del b

    n = len(tris)
    mean_build = sum(build_ms) / len(build_ms)
    mean_e2e = sum(e2e_ms) / len(e2e_ms)
    mean_build, mean_e2e, mean_prim, mean_bounce = max_over_ranks(
        [mean_build, mean_e2e, sum(prim_ms) / len(prim_ms), sum(bounce_ms) / len(bounce_ms)], dist, "cuda")
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    value = replica_rate(n, mean_build, world)
    e2e = replica_rate(n, mean_e2e, world)
    prim_rate = replica_rate(len(rays), mean_prim, world)
    bounce_rate = replica_rate(len(bounce), mean_bounce, world)

    arch = None if args.no_arch_scene else arch_scene(ctx, stream, max(3, args.steps // 4), args.warmup, flush)
    batch = None if args.no_batched else batched_scenes(G, ctx, BvhBuildParams.medium_build())
    served = None if args.no_serving else serving(BvhBuildParams.medium_build())

    # CPU baseline (the oracle on this host's cores, bounded sample): two full
    # builds, and the primary batch traced with node-visit / triangle-test
    # counters, which also give the traversal's algorithmic bytes.
    cores = os.cpu_count() or 1
    cpu_rate, cpu_t, cpu_trace = cpu_baseline(tris, p, rays, cores, ctx)

    peak, peak_kind = measured_peak()
    traffic_db = {}
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        traffic_db = json.load(open(tpath))

    # roofline of the build's dominant kernel (largest share of device time in
    # the event-bracketed build): algorithmic bytes per launch / mean launch
    # time; traffic = DRAM bytes per launch from the ncu capture (profiles/)
    models = kernel_byte_models(stats.leaf_count, stats.ploc_sum_counts, n_nodes, n_prims,
                                cpu_trace.get("search_nodes"))
    build_kernels = {}
    for k, v in kernel_profile.items():
        if k.startswith("k_traverse"):
            continue
        k = "k_find" if k.startswith("k_find") else k  # one search kernel, two launch forms
        a = build_kernels.setdefault(k, {"launches": 0, "total_ms": 0.0})
        a["launches"] += v["launches"]
        a["total_ms"] += v["total_ms"]
    ranked = sorted(build_kernels.items(), key=lambda kv: -kv[1]["total_ms"])
    dom_name, dom = next(((k, v) for k, v in ranked if models.get(k)), ranked[0])
    dom_launches = max(dom["launches"], 1)
    dom_bytes = models.get(dom_name, 0) / dom_launches
    dom_ms = dom["total_ms"] / dom_launches
    dom_achieved = dom_bytes / (dom_ms * 1e-3) / 1e9 if dom_ms > 0 else 0.0
    build_total_ms = sum(v["total_ms"] for v in build_kernels.values())

    # whole build against the same peak (the build is latency- and launch-bound)
    build_bytes = build_byte_model(stats.leaf_count, n, stats.ploc_sum_counts, n_nodes, n_prims)
    build_achieved = build_bytes / (mean_build * 1e-3) / 1e9

    # traversal: one launch per batch, timed above with CUDA events on the
    # library's stream.  Algorithmic bytes per ray: 32 (ray) + 8 (hit) + 80 per
    # node visited + 36 per triangle tested (visit/test counts: oracle)
    alg_bytes = 40.0 * len(rays) + 80.0 * cpu_trace["visits"] + 36.0 * cpu_trace["tests"]
    achieved = alg_bytes / (mean_prim * 1e-3) / 1e9

    line = {
        "metric": METRIC, "value": value, "unit": "Mtris/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mean_build, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded PCG64 clustered scene)",
        "config": {"workload": WORKLOAD, "n_tris": n, "preset": "slow_build", "leaves": stats.leaf_count,
                   "cwbvh_nodes": n_nodes, "primary_rays": len(rays), "bounce_rays": len(bounce),
                   "l2": "512 MB flush between timed steps", "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e, "unit": "Mtris/s", "h2d_bytes_per_step": n * 36,
                "d2h_bytes_per_step": n_nodes * 80 + n_prims * 4, "ms_per_step": mean_e2e},
        "traversal": {"primary_mrays_s": prim_rate, "bounce_mrays_s": bounce_rate, "primary_ms": mean_prim,
                      "bounce_ms": mean_bounce},
        "build_stages_ms": {"presplit": stats.stage_ms[0], "ploc": stats.stage_ms[1],
                            "reinsertion": stats.stage_ms[2], "cwbvh": stats.stage_ms[3]},
        "roofline": {"kernel": dom_name, "bound": "hbm", "achieved": dom_achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": dom_achieved / peak,
                     "traffic": traffic_db.get(dom_name), "algorithmic_bytes_per_launch": dom_bytes,
                     "launches": dom["launches"], "mean_launch_ms": dom_ms,
                     "share_of_build_kernel_time": dom["total_ms"] / build_total_ms if build_total_ms else None,
                     "note": ROOFLINE_NOTES.get(dom_name, "")},
        "roofline_build": {"bound": "hbm", "achieved": build_achieved, "peak": peak, "unit": "GB/s",
                           "frac": build_achieved / peak, "algorithmic_bytes": build_bytes,
                           "bytes_per_leaf": build_bytes / max(stats.leaf_count, 1)},
        "roofline_traversal": {"kernel": "k_traverse<closest> (primary batch)", "bound": "hbm",
                               "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                               "traffic": traffic_db.get("k_traverse_closest"),
                               "algorithmic_bytes_per_launch": alg_bytes, "bytes_per_ray": alg_bytes / len(rays)},
        "architectural_scene": arch,
        "batched": batch,
        "serving": served,
        "cpu_baseline": {"value": cpu_rate, "unit": "Mtris/s", "cores": cores, "kind": "port",
                         "sample": f"2 full {n}-triangle slow_build builds on {cores} threads "
                                   f"({sum(cpu_t):.1f} s)",
                         "primary_mrays_s": cpu_trace["mrays_s"]},
        "gpu_launches": launches,
        "kernel_profile_ms": {k: round(v["total_ms"], 4) for k, v in sorted(kernel_profile.items(),
                                                                             key=lambda kv: -kv[1]["total_ms"])},
        "clocks": clk,
        "wall_s_timed_builds": t_wall,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
