"""RtCompressedTriangle on the GPU vs the oracle, bit for bit: the 24-byte
records (f32 v0, half edges rounded to nearest even) and closest-hit /
occlusion traversal with RtCompressedTriangle::intersect."""
import numpy as np
import pytest

from oracle import oracle as O
from obvhs_gb300 import test_util as T
from obvhs_gb300.params import BvhBuildParams

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import obvhs_gb300 as g

    return g


def _tris(n, seed):
    """Triangles of edge up to ~0.8 with centroids in a cube of side 12."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-6, 6, size=(n, 1, 3))
    return (c + rng.uniform(-0.4, 0.4, size=(n, 3, 3))).reshape(-1, 9).astype(np.float32)


def _rays(n, seed, lo=-12, hi=12):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = T.uniform_sample_sphere(rng.random(n).astype(np.float32), rng.random(n).astype(np.float32))
    tmax = rng.uniform(0.5, 30, size=n).astype(np.float32)
    tmax[::3] = np.inf
    return T.make_rays(o, d, 0.0, tmax)


@pytest.mark.parametrize("n_tris,preset", [(60_000, "medium_build"), (300_000, "fast_build")])
def test_compressed_records_and_traversal_bitexact(G, n_tris, preset):
    tris = _tris(n_tris, n_tris)
    cw = G.build_cwbvh_from_tris(tris, getattr(BvhBuildParams, preset)())
    cw.set_triangles_compressed(tris)
    nodes, pidx = cw.download()
    ct = cw.download_compressed()
    assert np.array_equal(ct, O.compress_tris(tris, pidx))
    rays = _rays(50_000, n_tris)
    ids, t = cw.ray_traverse_compressed(rays)
    oids, ot = O.traverse_compressed(nodes, pidx, ct, rays, 0, nthreads=8)
    assert (oids != 0xFFFFFFFF).sum() > 1000
    assert np.array_equal(ids, oids) and np.array_equal(t.view(np.uint32), ot.view(np.uint32))
    miss = cw.ray_traverse_miss_compressed(rays)
    omiss, _ = O.traverse_compressed(nodes, pidx, ct, rays, 1, nthreads=8)
    assert np.array_equal(miss, omiss == 0xFFFFFFFF)
    assert miss.any() and (~miss).any()


def test_compressed_device_rays(G):
    import torch

    tris = _tris(20_000, 7)
    cw = G.build_cwbvh_from_tris(tris, BvhBuildParams.medium_build())
    cw.set_triangles_compressed(torch.from_numpy(tris).cuda())
    rays = _rays(10_000, 3)
    ids, t = cw.ray_traverse_compressed(rays)
    dev = cw.ray_traverse_compressed(torch.from_numpy(rays).cuda()).cpu().numpy().view(np.uint32)
    assert np.array_equal(dev[:, 0], ids) and np.array_equal(dev[:, 1], t.view(np.uint32))
