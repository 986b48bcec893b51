"""The serving loop's scheduling on the CPU: admission by budget, LRU
eviction with pins, rebuilds after eviction, continuous batching, and
results that are the same alone and in the mix (a CPU fake backend)."""
import numpy as np
import pytest

from obvhs_gb300 import serve


class FakeBackend:
    """Handles are (scene digest, size); a ray's result depends only on its
    scene and its own data, like a real traversal."""

    def __init__(self, delay=0.0):
        self.builds = []   # sizes of every build step
        self.traces = []   # requests per trace step
        self.freed = 0
        self.delay = delay

    def estimate_bytes(self, n):
        return 100 * int(n)

    def bytes_of(self, h):
        return 100 * h[1]

    def free(self, h):
        self.freed += 1

    def _h(self, tris):
        return (float(np.asarray(tris, np.float64).sum()), len(tris))

    def build_many(self, tris_list):
        import time

        time.sleep(self.delay)
        self.builds.append(len(tris_list))
        return [self._h(t) for t in tris_list]

    def build_one(self, tris):
        return self.build_many([tris])[0]

    @staticmethod
    def _trace(h, rays):
        ids = (np.floor(np.abs(rays[:, 0] * 1000 + h[0])) % 997).astype(np.uint32)
        return ids, rays[:, 3] + np.float32(h[1])

    def trace_many(self, items):
        import time

        time.sleep(self.delay)
        self.traces.append(len(items))
        res = []
        for it in items:
            ids, t = self._trace(it[0], it[1])
            out = it[2] if len(it) > 2 else None
            if out is not None:  # the client's (n, 2) uint32 buffer
                out[:, 0] = ids
                out[:, 1] = t.astype(np.float32).view(np.uint32)
                res.append(out)
            else:
                res.append((ids, t))
        return res

    def trace_one(self, h, r, out=None):
        return self.trace_many([(h, r, out)])[0]


def _pools(rng, k=4):
    tris = [rng.random((500, 9), dtype=np.float32) for _ in range(k)]
    rays = [(rng.random((300, 8), dtype=np.float32), rng.random((300, 8), dtype=np.float32)) for _ in range(k)]
    return tris, rays


def _stream(seed, n=300, rate=20_000.0, preloaded=2):
    rng = np.random.default_rng(seed)
    tris, rays = _pools(rng)
    reqs, scene_of = serve.make_stream(n, rate, tris, rays, rng, tri_range=(50, 500), ray_range=(10, 300),
                                       preloaded=preloaded)
    pre = [(i, tris[scene_of[i]][:100]) for i in range(preloaded)]
    return reqs, scene_of, pre, tris


def _check_alone(reqs, pre, backend):
    """Every ray batch's result equals its BVH's scene traced alone."""
    src = {i: t for i, t in pre}
    src.update({r.bvh_id: r.tris for r in reqs if r.kind == "build"})
    for r in reqs:
        assert r.done is not None and r.done >= r.arrival
        if r.kind == "rays":
            ids, t = backend._trace(backend._h(src[r.bvh_id]), r.rays)
            assert np.array_equal(r.result[0], ids) and np.array_equal(r.result[1], t)


def test_stream_shape():
    reqs, scene_of, _, _ = _stream(1, n=2000)
    kinds = np.array([r.kind == "build" for r in reqs])
    assert 0.07 < kinds.mean() < 0.13
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) >= 0)
    gaps = np.diff(arr)
    assert abs(gaps.mean() * 20_000 - 1) < 0.1  # Poisson at the given rate
    for r in reqs:
        if r.kind == "rays":
            assert r.bvh_id < len(scene_of)


def test_continuous_server_batches_and_matches_alone():
    reqs, _, pre, _ = _stream(2)
    b = FakeBackend(delay=0.002)
    s = serve.ContinuousServer(b, budget=10**9)
    s.run(reqs, preload=pre)
    _check_alone(reqs, pre, b)
    # continuous batching: far fewer launches than requests
    assert len(b.traces) < sum(r.kind == "rays" for r in reqs) / 2
    summ = serve.summarize(reqs)
    assert summ["latency_rays"]["p99_ms"] >= summ["latency_rays"]["p50_ms"]


def test_summary_pools_the_latencies_of_earlier_runs():
    """Percentiles over several runs of one stream count every request of
    every run; throughput and span are the last run's."""
    reqs = [serve.Request(i, "rays", 0.001 * i, 0, rays=np.zeros((10, 8), np.float32)) for i in range(100)]
    for r in reqs:
        r.done = r.arrival + 0.001
    first = serve.snapshot(reqs)
    reqs[0].done = reqs[0].arrival + 1.0  # one stall in the last run
    alone = serve.summarize(reqs)
    pooled = serve.summarize(reqs, [first, first])
    assert pooled["runs"] == 3 and alone["runs"] == 1
    assert pooled["span_s"] == alone["span_s"] and pooled["mrays_s"] == alone["mrays_s"]
    assert alone["latency_rays"]["max_ms"] == pooled["latency_rays"]["max_ms"] > 999
    # 1 slow request of 100 sets the p99 of one run, not of 300 requests
    assert alone["latency_rays"]["p99_ms"] > 10
    assert pooled["latency_rays"]["p99_ms"] < 1.5


def test_plain_server_one_call_per_request():
    reqs, _, pre, _ = _stream(3, n=120)
    b = FakeBackend()
    serve.PlainServer(b, budget=10**9).run(reqs, preload=pre)
    _check_alone(reqs, pre, b)
    assert all(n == 1 for n in b.builds) and all(n == 1 for n in b.traces)
    assert len(b.traces) == sum(r.kind == "rays" for r in reqs)


@pytest.mark.parametrize("server", ["continuous", "plain"])
def test_client_hit_buffers(server):
    """Requests that bring their own hit buffer get their hits there, the
    same as without one; the others still get copies."""
    reqs, _, pre, _ = _stream(6, n=200)
    for k, r in enumerate(reqs):
        if r.kind == "rays" and k % 2 == 0:
            r.out = np.zeros((len(r.rays), 2), np.uint32)
    b = FakeBackend()
    cls = serve.ContinuousServer if server == "continuous" else serve.PlainServer
    cls(b, budget=10**9).run(reqs, preload=pre)
    _check_alone(reqs, pre, b)
    for r in reqs:
        if r.out is not None:
            assert np.shares_memory(r.result[0], r.out)


@pytest.mark.parametrize("server", ["continuous", "plain"])
def test_small_budget_evicts_lru_and_rebuilds(server):
    reqs, _, pre, _ = _stream(4, n=300)
    b = FakeBackend(delay=0.0005)
    budget = 100 * 1200  # room for two or three scenes
    s = serve.ContinuousServer(b, budget) if server == "continuous" else serve.PlainServer(b, budget)
    s.run(reqs, preload=pre)
    _check_alone(reqs, pre, b)
    assert s.store.evictions > 0 and b.freed == s.store.evictions
    assert s.store.bytes <= budget
    assert s.rebuilds > 0


def test_store_never_evicts_pinned():
    st = serve.ResidentStore(300)
    freed = []
    st.add(1, "a", 100)
    st.add(2, "b", 100)
    st.add(3, "c", 100)
    st.pin(1)
    st.get(2)  # 2 becomes most recent: 3 is the LRU unpinned one
    assert st.make_room(100, freed.append)
    assert freed == ["c"] and 1 in st and 2 in st
    st.pin(2)
    assert not st.make_room(250, freed.append)  # only pinned ones left to evict
    assert freed == ["c"]


def test_oversized_build_raises():
    reqs, _, pre, _ = _stream(5, n=50)
    b = FakeBackend()
    with pytest.raises(MemoryError):
        serve.ContinuousServer(b, budget=1000).run(reqs, preload=[])
