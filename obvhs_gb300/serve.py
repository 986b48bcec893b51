"""Serving: a request loop over resident BVHs, with continuous batching.

The reference has no serving layer; this module is the serving form of its
hot path.  Two kinds of request arrive over time:

  build  a scene's triangles (host f32, n x 9)  ->  a resident BVH (its id)
  rays   a resident BVH's id and a ray batch (host f32, n x 8)
         ->  closest hits (primitive id, t), as CwBvh::ray_traverse gives them

ContinuousServer keeps built BVHs resident on the device and admits work by
an HBM budget: a build is admitted when the resident BVHs plus its estimated
size fit, after evicting least-recently-used BVHs that no queued or running
ray batch needs; a ray batch is admitted while the rays of the running step
stay under a cap.  Two workers overlap on the GPU, each on its own context
(CUDA stream): the builder takes every queued build at once into one
segmented build, the tracer takes every queued ray batch whose BVH is
resident into one multi-BVH traversal launch.  Requests that arrive while a
step runs join the next one, so new work keeps entering as slots and memory
free up.  A ray batch for an evicted BVH has it rebuilt from the retained
triangles.

PlainServer is the baseline: one request per call, in arrival order (a build
call per scene, a traversal call per ray batch), under the same budget.

Latency is arrival to result on the host.  A ray request may carry the
client's own hit buffer (Request.out, pinned): the hits are copied straight
into it and the request is done when they have landed; otherwise the server
copies them out of its step buffer.  Backends: GpuBackend (this library) and
any object with the same four methods (tests use a CPU fake).
"""
from __future__ import annotations

import dataclasses
import threading
import time
from collections import OrderedDict

import numpy as np


@dataclasses.dataclass
class Request:
    rid: int
    kind: str                 # "build" or "rays"
    arrival: float            # seconds from the start of the run
    bvh_id: int               # build: the id it creates; rays: the id it targets
    tris: np.ndarray | None = None
    rays: np.ndarray | None = None
    done: float | None = None
    result: object = None
    step: int = -1            # the step (launch) that served it
    out: np.ndarray | None = None  # rays: the client's (n, 2) uint32 hit buffer; pinned, the hits are copied straight in


class ResidentStore:
    """Resident BVHs by id, least recently used first, with pins (held by
    queued and running ray batches) that exclude a BVH from eviction."""

    def __init__(self, budget: int):
        self.budget = int(budget)
        self.items = OrderedDict()  # id -> (handle, bytes)
        self.bytes = 0
        self.pins = {}
        self.evictions = 0

    def __contains__(self, bvh_id):
        return bvh_id in self.items

    def get(self, bvh_id):
        self.items.move_to_end(bvh_id)
        return self.items[bvh_id][0]

    def add(self, bvh_id, handle, nbytes: int):
        self.items[bvh_id] = (handle, int(nbytes))
        self.bytes += int(nbytes)

    def pin(self, bvh_id):
        self.pins[bvh_id] = self.pins.get(bvh_id, 0) + 1

    def unpin(self, bvh_id):
        self.pins[bvh_id] -= 1
        if not self.pins[bvh_id]:
            del self.pins[bvh_id]

    def make_room(self, nbytes: int, free) -> bool:
        """Evicts unpinned BVHs, least recently used first, until nbytes more
        fit; False (nothing evicted beyond need) if they cannot."""
        if self.bytes + nbytes <= self.budget:
            return True
        evictable = sum(b for k, (_, b) in self.items.items() if k not in self.pins)
        if self.bytes - evictable + nbytes > self.budget:
            return False
        for k in list(self.items):
            if self.bytes + nbytes <= self.budget:
                break
            if k in self.pins:
                continue
            h, b = self.items.pop(k)
            self.bytes -= b
            self.evictions += 1
            free(h)
        return True


class _Base:
    def __init__(self, backend, budget: int, result_sink=None):
        self.backend = backend
        self.store = ResidentStore(budget)
        self.sources = {}  # bvh id -> triangles, for rebuilds after eviction
        self.rebuilds = 0
        self.sink = result_sink  # maps a ray batch's (ids, t) to what the request keeps (default: all of it)

    def _keep(self, result, r=None):
        """What a ray request keeps: the sink's value, else (ids, t) views of
        the client's own hit buffer when it gave one, else the backend's own
        copy of the hits (results may be views of a reused buffer)."""
        if r is not None and r.out is not None:
            if self.sink:
                return self.sink(r.out)
            return r.out[:, 0], r.out[:, 1].view(np.float32)
        if self.sink:
            return self.sink(result)
        own = getattr(self.backend, "result", None)
        return own(result) if own else result

    def _free(self, h):
        self.backend.free(h)


class PlainServer(_Base):
    """One request per call, in arrival order."""

    def run(self, requests, preload=()):
        for bvh_id, tris in preload:
            self._build(bvh_id, tris)
        t0 = time.perf_counter()
        for step, r in enumerate(sorted(requests, key=lambda q: q.arrival)):
            wait = r.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            if r.kind == "build":
                self.sources[r.bvh_id] = r.tris
                self._build(r.bvh_id, r.tris)
                r.result = r.bvh_id
            else:
                if r.bvh_id not in self.store:
                    self.rebuilds += 1
                    self._build(r.bvh_id, self.sources[r.bvh_id])
                res = self.backend.trace_one(self.store.get(r.bvh_id), r.rays, r.out)
            r.done = time.perf_counter() - t0
            if r.kind == "rays":
                r.result = self._keep(res, r)
            r.step = step
        return requests

    def _build(self, bvh_id, tris):
        self.sources[bvh_id] = tris
        if not self.store.make_room(self.backend.estimate_bytes(len(tris)), self._free):
            raise MemoryError("a build does not fit the HBM budget")
        h = self.backend.build_one(tris)
        self.store.add(bvh_id, h, self.backend.bytes_of(h))


class ContinuousServer(_Base):
    """Continuous batching: a builder and a tracer worker, one launch per step
    each, overlapping on the device."""

    def __init__(self, backend, budget: int, max_step_rays: int = 1 << 25, max_step_tris: int = 1 << 25,
                 max_wait: float = 0.0, result_sink=None):
        super().__init__(backend, budget, result_sink)
        self.max_step_rays = max_step_rays
        self.max_step_tris = max_step_tris
        self.max_wait = max_wait  # optional hold to let a step fill (0: launch as soon as work is there)
        self.cv = threading.Condition()
        self.steps = {"build": 0, "rays": 0}

    def run(self, requests, preload=()):
        for bvh_id, tris in preload:
            self.sources[bvh_id] = tris
        if preload:
            hs = self.backend.build_many([t for _, t in preload])
            for (bvh_id, _), h in zip(preload, hs):
                self.store.add(bvh_id, h, self.backend.bytes_of(h))
        self.pending = sorted(requests, key=lambda q: q.arrival)
        self.next_arrival = 0
        self.builds = []       # admitted build requests (and rebuild markers)
        self.rays = []         # admitted ray requests
        self.building = set()  # ids of BVHs being built
        self.left = len(requests)
        self.error = None
        self.t0 = time.perf_counter()
        workers = [threading.Thread(target=self._guard, args=(self._builder,)),
                   threading.Thread(target=self._guard, args=(self._tracer,))]
        for w in workers:
            w.start()
        for w in workers:
            w.join()
        if self.error:
            raise self.error
        return requests

    # -- shared state (under self.cv) ------------------------------------

    def _now(self):
        return time.perf_counter() - self.t0

    def _admit_arrivals(self):
        now = self._now()
        while self.next_arrival < len(self.pending) and self.pending[self.next_arrival].arrival <= now:
            r = self.pending[self.next_arrival]
            self.next_arrival += 1
            if r.kind == "build":
                self.sources[r.bvh_id] = r.tris
                self.builds.append(r)
            else:
                self.store.pin(r.bvh_id)  # queued: not evictable
                self.rays.append(r)

    def _wait(self):
        """Sleeps until the next arrival or a notification."""
        timeout = 0.05
        if self.next_arrival < len(self.pending):
            timeout = max(0.0, min(timeout, self.pending[self.next_arrival].arrival - self._now()))
        self.cv.wait(timeout)

    def _finish(self, r, result, step, done=None):
        r.result = result
        r.done = self._now() if done is None else done
        r.step = step
        self.left -= 1

    def _guard(self, fn):
        try:
            fn()
        except BaseException as e:  # surfaced by run()
            with self.cv:
                self.error = e
                self.left = 0
                self.cv.notify_all()

    # -- workers -----------------------------------------------------------

    def _builder(self):
        while True:
            with self.cv:
                while True:
                    if self.left <= 0:
                        return
                    self._admit_arrivals()
                    # ray batches whose BVH was evicted: rebuild from the source
                    for r in self.rays:
                        if r.bvh_id not in self.store and r.bvh_id not in self.building and \
                                not any(b.bvh_id == r.bvh_id for b in self.builds) and r.bvh_id in self.sources:
                            self.builds.append(Request(-1, "build", r.arrival, r.bvh_id, self.sources[r.bvh_id]))
                            self.rebuilds += 1
                    take, tris = [], 0
                    for b in self.builds:
                        if take and tris + len(b.tris) > self.max_step_tris:
                            break
                        if not self.store.make_room(self.backend.estimate_bytes(tris + len(b.tris)), self._free):
                            break
                        take.append(b)
                        tris += len(b.tris)
                    if take:
                        break
                    if self.builds and not self.store.items and not self.building:
                        raise MemoryError("a build does not fit the HBM budget")
                    self._wait()
                self.builds = self.builds[len(take):]
                for b in take:
                    self.building.add(b.bvh_id)
                step = self.steps["build"]
                self.steps["build"] += 1
            hs = self.backend.build_many([b.tris for b in take])
            with self.cv:
                for b, h in zip(take, hs):
                    self.store.add(b.bvh_id, h, self.backend.bytes_of(h))
                    self.building.discard(b.bvh_id)
                    if b.rid >= 0:
                        self._finish(b, b.bvh_id, step)
                self.cv.notify_all()

    def _tracer(self):
        while True:
            with self.cv:
                while True:
                    if self.left <= 0:
                        return
                    self._admit_arrivals()
                    ready = [r for r in self.rays if r.bvh_id in self.store]
                    if ready and self.max_wait > 0 and self.next_arrival < len(self.pending):
                        # optional hold: wait for more work unless the oldest has waited long enough
                        if self._now() - ready[0].arrival < self.max_wait:
                            self._wait()
                            continue
                    if ready:
                        break
                    self._wait()
                take, n = [], 0
                for r in ready:
                    if take and n + len(r.rays) > self.max_step_rays:
                        break
                    take.append(r)
                    n += len(r.rays)
                ids = {id(r) for r in take}
                self.rays = [r for r in self.rays if id(r) not in ids]
                items = [(self.store.get(r.bvh_id), r.rays, r.out) for r in take]
                step = self.steps["rays"]
                self.steps["rays"] += 1
            results = self.backend.trace_many(items)
            done = self._now()
            kept = [self._keep(res, r) for r, res in zip(take, results)]
            with self.cv:
                for r, res in zip(take, kept):
                    self.store.unpin(r.bvh_id)
                    self._finish(r, res, step, done)
                self.cv.notify_all()


# --- the GPU backend -----------------------------------------------------------


def pinned_empty(shape, dtype) -> np.ndarray:
    """A numpy array in page-locked host memory (its copies to and from the
    device are asynchronous DMA, with no staging copy)."""
    import torch

    nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
    return torch.empty(max(nbytes, 1), dtype=torch.uint8, pin_memory=True).numpy()[:nbytes].view(dtype).reshape(shape)


def _is_pinned(a: np.ndarray) -> bool:
    import torch

    return a.flags.c_contiguous and torch.from_numpy(a).is_pinned()


class _Grow:
    """Grow-only buffer: pinned host memory or device memory."""

    def __init__(self, device=None):
        self.buf = None
        self.device = device

    def get(self, nbytes: int):
        import torch

        if self.buf is None or self.buf.numel() < nbytes:
            n = max(nbytes, 1 << 20) * 5 // 4
            if self.device is None:
                self.buf = torch.empty(n, dtype=torch.uint8, pin_memory=True)
            else:
                self.buf = torch.empty(n, dtype=torch.uint8, device=self.device)
        return self.buf[:nbytes]


class GpuBackend:
    """Builds and traversals through this library: a build context and a
    trace context (two CUDA streams).  Inputs in pinned host memory are copied
    to the device directly by the library (one asynchronous copy per request);
    other triangle inputs go through a pinned staging buffer first.  A step's
    hits come back into one pinned buffer, one copy per request:
    trace_many returns views of it (valid until the next step), result()
    copies one out."""

    def __init__(self, params, device: int = 0, bytes_per_tri_estimate: int = 96):
        from . import bvh

        self.G = bvh
        self.params = params
        self.bctx = bvh.Context(device)
        self.tctx = bvh.Context(device)
        self.per_tri = bytes_per_tri_estimate
        self.pin_build, self.pin_out = _Grow(), _Grow()

    def close(self):
        self.bctx.close()
        self.tctx.close()

    # sizes
    def estimate_bytes(self, n_tris: int) -> int:
        return int(n_tris) * self.per_tri

    @staticmethod
    def bytes_of(h) -> int:
        nn, npr, _ = h.info()
        return nn * 80 + npr * (4 + 64)

    def free(self, h):
        h.free()

    # builds
    def _stage_tris(self, tris_list):
        if all(_is_pinned(t) for t in tris_list):
            return tris_list
        total = sum(len(t) for t in tris_list) * 36
        buf = self.pin_build.get(total).numpy()
        views, at = [], 0
        for t in tris_list:
            nb = len(t) * 36
            v = buf[at:at + nb].view(np.float32).reshape(-1, 9)
            np.copyto(v, t)
            views.append(v)
            at += nb
        return views

    def build_many(self, tris_list):
        return self.G.build_cwbvh_from_tris_segmented(self._stage_tris(tris_list), self.params, ctx=self.bctx)

    def build_one(self, tris):
        return self.G.build_cwbvh_from_tris(self._stage_tris([tris])[0], self.params, ctx=self.bctx)

    # traversal
    def trace_many(self, items):
        """items: (handle, rays) or (handle, rays, out): hits go to `out`
        (the client's buffer) when given, else to the step buffer."""
        items = [(it[0], it[1], it[2] if len(it) > 2 else None) for it in items]
        n = sum(len(r) for _, r, o in items if o is None)
        out = self.pin_out.get(max(n, 1) * 8).numpy().view(np.uint32).reshape(-1, 2)
        index, bvhs, which, outs, at = {}, [], [], [], 0
        for h, r, o in items:
            k = index.setdefault(id(h), len(bvhs))
            if k == len(bvhs):
                bvhs.append(h)
            which.append(k)
            if o is None:
                o = out[at:at + len(r)]
                at += len(r)
            outs.append(o)
        self.G.ray_traverse_batches(bvhs, which, [r for _, r, _ in items], outs=outs, ctx=self.tctx)
        return outs

    def trace_one(self, h, r, out=None):
        return self.trace_many([(h, r, out)])[0]

    @staticmethod
    def result(block):
        """(primitive ids, t) of one request's hits, copied out."""
        return block[:, 0].copy(), block[:, 1].copy().view(np.float32)


# --- request streams and summaries -----------------------------------------------


def make_stream(n_requests: int, rate: float, scene_pool, ray_pool, rng, build_fraction: float = 0.1,
                tri_range=(10_000, 2_000_000), ray_range=(1_000, 1_000_000), zipf_s: float = 1.1, preloaded: int = 0):
    """Poisson arrivals at `rate` per second.  Builds take the first n
    triangles (log-uniform over tri_range) of a pooled scene; ray batches take
    the first n rays (log-uniform over ray_range) of the pooled primary or
    incoherent batch of their target's scene, the target chosen by Zipf(s)
    over the BVHs built so far, most recent first (ids 0..preloaded-1 exist
    before the first request).  scene_pool[k]: triangles; ray_pool[k]:
    (primary rays, incoherent rays) of scene k.  Returns (requests, the scene
    index of every BVH id)."""
    t = np.cumsum(rng.exponential(1.0 / rate, size=n_requests))
    scene_of = [k % len(scene_pool) for k in range(preloaded)]
    reqs = []
    for i in range(n_requests):
        if rng.random() < build_fraction or not scene_of:
            k = int(rng.integers(len(scene_pool)))
            n = int(np.exp(rng.uniform(np.log(tri_range[0]), np.log(tri_range[1]))))
            n = min(n, len(scene_pool[k]))
            reqs.append(Request(i, "build", float(t[i]), len(scene_of), tris=scene_pool[k][:n]))
            scene_of.append(k)
        else:
            ids = len(scene_of)
            w = 1.0 / np.arange(1, ids + 1) ** zipf_s
            rank = int(rng.choice(ids, p=w / w.sum()))
            target = ids - 1 - rank
            prim, inco = ray_pool[scene_of[target]]
            src = prim if rng.random() < 0.5 else inco
            n = int(np.exp(rng.uniform(np.log(ray_range[0]), np.log(ray_range[1]))))
            reqs.append(Request(i, "rays", float(t[i]), target, rays=src[:min(n, len(src))]))
    return reqs, scene_of


def snapshot(requests) -> list:
    """(kind, latency in s) of every request of a finished run."""
    return [(r.kind, r.done - r.arrival) for r in requests]


def summarize(requests, earlier=()) -> dict:
    """Throughput and latency of a finished run.  `earlier`: snapshots of
    earlier runs of the same stream, whose latencies join the percentiles
    (throughput and span are this run's)."""
    def pct(v):
        if not len(v):
            return {}
        v = np.asarray(v) * 1e3
        return {"p50_ms": float(np.percentile(v, 50)), "p99_ms": float(np.percentile(v, 99)),
                "p999_ms": float(np.percentile(v, 99.9)), "mean_ms": float(v.mean()), "max_ms": float(v.max())}

    rays = [r for r in requests if r.kind == "rays"]
    builds = [r for r in requests if r.kind == "build"]
    first = min(r.arrival for r in requests)
    last = max(r.done for r in requests)
    n_rays = sum(len(r.rays) for r in rays)
    n_tris = sum(len(r.tris) for r in builds)
    return {"requests": len(requests), "ray_requests": len(rays), "build_requests": len(builds),
            "rays": int(n_rays), "triangles_built": int(n_tris), "span_s": last - first,
            "mrays_s": n_rays / (last - first) / 1e6, "build_mtris_s": n_tris / (last - first) / 1e6,
            "latency_rays": pct([r.done - r.arrival for r in rays] + [l for s in earlier for k, l in s if k == "rays"]),
            "latency_builds": pct([r.done - r.arrival for r in builds] +
                                  [l for s in earlier for k, l in s if k == "build"]),
            "latency_all": pct([r.done - r.arrival for r in requests] + [l for s in earlier for _, l in s]),
            "launch_steps": len({(r.kind, r.step) for r in requests}), "runs": 1 + len(earlier)}


def clustered_pools(n_scenes: int, max_tris: int, max_rays: int, seed: int = 1005, pin: bool = True):
    """Pooled inputs of the clustered workload: n_scenes scenes of max_tris
    triangles (the clustered generator, seed offset k), and per scene
    max_rays primary rays (a square pinhole image from (0, 0, -35) looking
    along +z, 60 degree field of view) and max_rays incoherent rays (origins
    uniform in [-10, 10]^3, directions uniform on the sphere).  Prefixes of
    these are valid inputs of every smaller size.  pin: in page-locked host
    memory, as a serving front end would hand them over."""
    from . import scenes as S
    from . import test_util as T

    def pinned(a):
        if not pin:
            return a
        p = pinned_empty(a.shape, a.dtype)
        np.copyto(p, a)
        return p

    rng = np.random.default_rng(seed)
    side = int(np.ceil(np.sqrt(max_rays)))
    primary = pinned(S.pinhole_rays(side, side, (0.0, 0.0, -35.0), 60.0)[:max_rays])
    tris, rays = [], []
    for k in range(n_scenes):
        tris.append(pinned(S.scene2_tris(max_tris, offset=k)))
        o = rng.uniform(-10, 10, size=(max_rays, 3)).astype(np.float32)
        d = T.uniform_sample_sphere(rng.random(max_rays).astype(np.float32), rng.random(max_rays).astype(np.float32))
        rays.append((primary, pinned(T.make_rays(o, d, 0.0, np.inf))))
    return tris, rays
