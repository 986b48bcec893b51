"""Full builds at the benchmark's scale vs the oracle, bit for bit (needs a GPU).

The small cases in test_gpu_parity.py run every kernel in its single-tile or
single-block form.  These sizes exercise the forms that only large inputs
reach: PLOC passes with several tiles per block group and adaptive tile
sizes, reinsertion passes resolved by the whole grid, the persistent
reinsertion search, multi-wave radix sorts.  Each build is repeated to catch
races that make results depend on timing.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from obvhs_gb300 import scenes as S
from obvhs_gb300.params import PRESETS

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


@pytest.fixture(scope="module")
def G():
    import obvhs_gb300 as g

    return g


def _bytes_equal(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and a.tobytes() == b.tobytes()


@pytest.mark.parametrize("preset,n", [("slow", 1_000_000), ("fastest", 1_000_000),
                                      ("medium", 2_000_000)])
def test_clustered_scene_bitexact_repeated(G, preset, n):
    tris = S.scene2_tris(n)
    p = PRESETS[preset]()
    ob = O.build(tris=tris, params=p, nthreads=THREADS, keep_intermediate=False)
    for _ in range(3):
        cw = G.build_cwbvh_from_tris(tris, p)
        nodes, prims = cw.download()
        assert cw.stats.reinsertions == ob.reinsertions
        assert _bytes_equal(nodes, ob.cw_nodes)
        assert _bytes_equal(prims, ob.cw_pidx)


def test_ploc_one_million_u64(G):
    tris = S.scene2_tris(1_000_000).reshape(-1, 3, 3)
    aabbs = np.concatenate([tris.min(1), tris.max(1)], 1).astype(np.float32)
    on, op, omd, _ = O.ploc(aabbs, None, 14, 0, 0, nthreads=THREADS)
    b = G.PlocBuilder().build_ploc(14, aabbs, None, 0, 0)
    nodes, pidx = b.download()
    assert _bytes_equal(nodes, on)
    assert _bytes_equal(pidx, op)


def test_architectural_scene_build_and_rays_bitexact(G):
    """The 8M-triangle architectural generator at 2M: plain PLOC -> CWBVH
    (radius 14, distance 1 for 3 passes, U64), then incoherent closest-hit
    and shadow rays, all against the oracle."""
    from obvhs_gb300.params import BvhBuildParams

    tris = S.scene3_tris(2_000_000)
    closest, shadow = S.scene3_rays(200_000)
    p = BvhBuildParams(False, 14, 3, 0.0, 0.0, 0, 3, 3.0)
    ob = O.build(tris=tris, params=p, nthreads=THREADS, keep_intermediate=False)
    cw = G.build_cwbvh_from_tris(tris, p)
    nodes, prims = cw.download()
    assert _bytes_equal(nodes, ob.cw_nodes)
    assert _bytes_equal(prims, ob.cw_pidx)
    gid, gt = cw.ray_traverse(closest)
    oid, ot, _ = O.traverse(ob.cw_nodes, ob.cw_pidx, tris, closest, 0, nthreads=THREADS)
    assert np.array_equal(gid, oid)
    assert np.array_equal(gt.view(np.uint32), ot.view(np.uint32))
    gmiss = cw.ray_traverse_miss(shadow)
    omiss, _, _ = O.traverse(ob.cw_nodes, ob.cw_pidx, tris, shadow, 1, nthreads=THREADS)
    assert np.array_equal(gmiss, omiss == 0xFFFFFFFF)


def test_architectural_scene_full_size_bitexact(G):
    """The benchmark's headline workload at its full size: the 8M-triangle
    scene built PLOC -> CWBVH (radius 14, distance 1 for 3 passes, U64), the
    CWBVH bytes and primitive indices, every one of the 16M incoherent
    closest-hit rays (ids and t) and of the 16M shadow rays against the oracle
    (src/cwbvh/mod.rs:169-225)."""
    from obvhs_gb300.params import BvhBuildParams

    tris = S.scene3_tris(8_000_000)
    p = BvhBuildParams(False, 14, 3, 0.0, 0.0, 0, 3, 3.0)
    ob = O.build(tris=tris, params=p, nthreads=THREADS, keep_intermediate=False)
    cw = G.build_cwbvh_from_tris(tris, p)
    nodes, prims = cw.download()
    assert _bytes_equal(nodes, ob.cw_nodes)
    assert _bytes_equal(prims, ob.cw_pidx)
    del nodes, prims
    closest, shadow = S.scene3_rays(16_000_000)
    gid, gt = cw.ray_traverse(closest)
    oid, ot, _ = O.traverse(ob.cw_nodes, ob.cw_pidx, tris, closest, 0, nthreads=THREADS)
    assert (oid != 0xFFFFFFFF).mean() > 0.5
    assert np.array_equal(gid, oid)
    assert np.array_equal(gt.view(np.uint32), ot.view(np.uint32))
    del gid, gt, oid, ot, closest
    gmiss = cw.ray_traverse_miss(shadow)
    omiss, _, _ = O.traverse(ob.cw_nodes, ob.cw_pidx, tris, shadow, 1, nthreads=THREADS)
    assert np.array_equal(gmiss, omiss == 0xFFFFFFFF)
    assert gmiss.any() and (~gmiss).any()
