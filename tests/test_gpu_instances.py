"""Instance traversal (CwBvh::ray_traverse_tlas_blas) on the GPU vs the
oracle, bit for bit: geometry id, BVH-order primitive id, original id, t."""
import numpy as np
import pytest

from oracle import oracle as O
from obvhs_gb300.params import BvhBuildParams

import instances as I

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import obvhs_gb300 as g

    return g


@pytest.mark.parametrize("n_blas,tlas_prims", [(1, 3), (12, 1), (40, 3)])
def test_tlas_blas_bitexact(G, n_blas, tlas_prims):
    blas_tris = I.instanced_scene(n_blas, seed=n_blas)
    blas = [G.build_cwbvh_from_tris(t, BvhBuildParams.medium_build()) for t in blas_tris]
    tlas = G.build_cwbvh(I.instance_boxes(blas_tris), I.tlas_params(tlas_prims))
    rays = I.incoherent_rays(60_000, seed=n_blas + 1)
    g, p, orig, t = tlas.ray_traverse_tlas_blas(blas, rays)
    tn, tp = tlas.download()
    ob = [(b.download()[0], b.download()[1], tr) for b, tr in zip(blas, blas_tris)]
    og, op, oo, ot = O.traverse_tlas(tn, tp, ob, rays, nthreads=8)
    assert (og != 0xFFFFFFFF).sum() > 1000
    assert np.array_equal(g, og) and np.array_equal(p, op) and np.array_equal(orig, oo)
    assert np.array_equal(t.view(np.uint32), ot.view(np.uint32))


def test_tlas_blas_device_rays(G):
    import torch

    blas_tris = I.instanced_scene(6, seed=11)
    blas = [G.build_cwbvh_from_tris(t, BvhBuildParams.fast_build()) for t in blas_tris]
    tlas = G.build_cwbvh(I.instance_boxes(blas_tris), I.tlas_params(3))
    rays = I.incoherent_rays(20_000, seed=12)
    host = tlas.ray_traverse_tlas_blas(blas, rays)
    dev = tlas.ray_traverse_tlas_blas(blas, torch.from_numpy(rays).cuda()).cpu().numpy().view(np.uint32)
    for k in range(4):
        assert np.array_equal(dev[:, k], host[k].view(np.uint32))
