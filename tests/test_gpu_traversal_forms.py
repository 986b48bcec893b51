"""Traversal launch forms (block size, group stack in local or shared memory)
give identical results, and the autotuner picks among them (needs a GPU).

The reference traverses with one 32-entry StackStack per ray
(src/cwbvh/mod.rs:60-64, src/faststack.rs:299-303); every form keeps its 32
entries and clamping, so hits are bit-identical, including for rays deep
enough to clamp."""
import numpy as np
import pytest

from obvhs_gb300 import scenes as S
from obvhs_gb300 import test_util as T
from obvhs_gb300.params import BvhBuildParams

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import obvhs_gb300 as g

    return g


def _rays(n, seed, lo, hi):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = T.uniform_sample_sphere(rng.random(n).astype(np.float32), rng.random(n).astype(np.float32))
    tmax = rng.uniform(0.5, 40, size=n).astype(np.float32)
    tmax[::2] = np.inf
    return T.make_rays(o, d, 0.0, tmax)


def test_every_form_gives_the_default_hits(G):
    import torch

    tris = S.scene3_tris(300_000)
    rays = _rays(200_000, 1, [-10, -3, -10], [10, 3, 10])
    ctx = G.Context()
    try:
        cw = G.build_cwbvh_from_tris(tris, BvhBuildParams.medium_build(), ctx=ctx)
        ref_ids, ref_t = cw.ray_traverse(rays)
        ref_miss = cw.ray_traverse_miss(rays)
        d_rays = torch.from_numpy(rays).cuda()
        owner = torch.zeros(len(rays), dtype=torch.int32, device="cuda")
        for block, smem in G.Context.TRAVERSAL_CONFIGS:
            ctx.set_traversal_config(block, smem)
            ids, t = cw.ray_traverse(rays)
            assert np.array_equal(ids, ref_ids), (block, smem)
            assert np.array_equal(t.view(np.uint32), ref_t.view(np.uint32)), (block, smem)
            assert np.array_equal(cw.ray_traverse_miss(rays), ref_miss), (block, smem)
            multi = G.ray_traverse_multi([cw], owner, d_rays, ctx=ctx).cpu().numpy().view(np.uint32)
            assert np.array_equal(multi[:, 0], ref_ids.view(np.uint32)), (block, smem)
            assert np.array_equal(multi[:, 1], ref_t.view(np.uint32)), (block, smem)
        ctx.set_traversal_config(0, False)
        ids, _ = cw.ray_traverse(rays)
        assert np.array_equal(ids, ref_ids)
    finally:
        ctx.close()


def test_invalid_forms_are_rejected(G):
    from obvhs_gb300._native import ObvhsError

    ctx = G.Context()
    try:
        for block, smem in ((32, False), (256, True), (100, False)):
            with pytest.raises(ObvhsError):
                ctx.set_traversal_config(block, smem)
    finally:
        ctx.close()


def test_autotuner_reports_radius_and_traversal_form(G):
    import torch
    from obvhs_gb300 import autotune as A

    scenes = [torch.from_numpy(S.scene2_tris(n, offset=i)).cuda() for i, n in enumerate((3000, 20_000, 60_000))]
    rays = [_rays(4096, 10 + i, [-12, -12, -12], [12, 12, 12]) for i in range(3)]
    owner = torch.from_numpy(np.concatenate([np.full(len(r), i, np.int32) for i, r in enumerate(rays)])).cuda()
    d_rays = torch.from_numpy(np.concatenate(rays)).cuda()
    p, tune = A.tune_segmented(scenes, d_rays, owner, BvhBuildParams.medium_build(), radii=(8, 14), reps=1)
    assert p.ploc_search_distance in (8, 14)
    assert set(tune["radius_s"]) == {8, 14}
    trav = tune["traversal"]
    assert (trav["block"], trav["smem_stack"]) in G.Context.TRAVERSAL_CONFIGS
    assert len(trav["ms"]) == len(G.Context.TRAVERSAL_CONFIGS)
