"""The batched workload at full size: 512 clustered scenes of 1k-200k
triangles (log-uniform, scene i from the clustered generator with seed offset
i; about 20M triangles), each with 4,096-262,144 incoherent rays in
proportion to its size (about 28M rays), built as one segmented batch and
traced in one multi-BVH launch.  Scenes spread over the size range, the
smallest and the largest among them, are compared with the oracle: CWBVH
nodes and primitive indices byte for byte, and every ray's hit id and t."""
import dataclasses

import numpy as np
import pytest

from oracle import oracle as O
from obvhs_gb300 import autotune as A
from obvhs_gb300 import scenes as S
from obvhs_gb300 import test_util as T
from obvhs_gb300.params import BvhBuildParams

pytestmark = pytest.mark.gpu


def _batch(n_scenes=512, seed=1004):
    """The scenes and rays of the batched benchmark workload (same seeds)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(1000), np.log(200_000), size=n_scenes)).astype(np.int64)
    tris, rays = [], []
    for i, n in enumerate(sizes):
        t = S.scene2_tris(int(n), offset=i)
        tris.append(t)
        k = int(4096 + (n - 1000) * (262_144 - 4096) / (200_000 - 1000))
        v = t.reshape(-1, 3)
        lo, hi = v.min(0), v.max(0)
        o = rng.uniform(lo, hi, size=(k, 3)).astype(np.float32)
        d = T.uniform_sample_sphere(rng.random(k).astype(np.float32), rng.random(k).astype(np.float32))
        rays.append(T.make_rays(o, d, 0.0, np.inf))
    return sizes, tris, rays


@pytest.mark.parametrize("radius", [8, 14])
def test_batched_workload_full_size_against_the_oracle(radius):
    import torch

    import obvhs_gb300 as G

    sizes, tris, rays = _batch()
    p = dataclasses.replace(BvhBuildParams.medium_build(), ploc_search_distance=radius)
    d_tris = [torch.from_numpy(t).cuda() for t in tris]
    owner = np.concatenate([np.full(len(r), i, np.int32) for i, r in enumerate(rays)])
    start = np.concatenate([[0], np.cumsum([len(r) for r in rays])])
    all_rays = torch.from_numpy(np.concatenate(rays)).cuda()
    bvhs = G.build_cwbvh_from_tris_segmented(d_tris, p)
    hits = G.ray_traverse_multi(bvhs, torch.from_numpy(owner).cuda(), all_rays)
    torch.cuda.synchronize()
    got = hits.cpu().numpy().view(np.uint32).reshape(-1, 2)
    pick = sorted(set(A.sample_indices(sizes, 18).tolist()) | {int(np.argmin(sizes)), int(np.argmax(sizes))})
    for i in pick:
        ob = O.build(tris=tris[i], params=p, nthreads=16, keep_intermediate=False)
        nodes, pidx = bvhs[i].download()
        assert nodes.tobytes() == ob.cw_nodes.tobytes(), f"scene {i} ({sizes[i]} triangles): nodes"
        assert pidx.tobytes() == ob.cw_pidx.tobytes(), f"scene {i}: primitive indices"
        ids, t, _ = O.traverse(ob.cw_nodes, ob.cw_pidx, tris[i], rays[i], 0, nthreads=16)
        mine = got[start[i]:start[i + 1]]
        assert np.array_equal(mine[:, 0], ids), f"scene {i}: hit ids"
        assert np.array_equal(mine[:, 1], t.view(np.uint32)), f"scene {i}: hit t"
    for b in bvhs:
        b.free()
