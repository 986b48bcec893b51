"""Instanced test scenes for the TLAS/BLAS traversal tests: a few BLAS of
uneven size (clustered-scene generator, shifted apart and partly
overlapping), a TLAS over their boxes, and incoherent rays through them."""
import numpy as np

from oracle import oracle as O
from obvhs_gb300 import test_util as T
from obvhs_gb300.params import BvhBuildParams


def instanced_scene(n_blas=12, seed=5, sizes=(500, 6000)):
    """Per BLAS: triangles with centroids in a cube of side 3 and vertex
    offsets up to 0.25, shifted by up to 5 so that instances partly overlap."""
    rng = np.random.default_rng(seed)
    blas_tris = []
    for b in range(n_blas):
        n = int(rng.integers(sizes[0], sizes[1]))
        c = rng.uniform(-1.5, 1.5, size=(n, 1, 3))
        v = c + rng.uniform(-0.25, 0.25, size=(n, 3, 3))
        shift = rng.uniform(-5, 5, size=(1, 1, 3))
        blas_tris.append((v + shift).reshape(-1, 9).astype(np.float32))
    return blas_tris


def instance_boxes(blas_tris):
    out = []
    for t in blas_tris:
        v = t.reshape(-1, 3)
        out.append(np.concatenate([v.min(0), v.max(0)]))
    return np.asarray(out, np.float32)


def incoherent_rays(n, seed=9):
    """Origins in a cube of side 16 around the instances; half the rays aim
    at random points among them, half go in uniform directions."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(-8, 8, size=(n, 3)).astype(np.float32)
    d = T.uniform_sample_sphere(rng.random(n).astype(np.float32), rng.random(n).astype(np.float32))
    aim = rng.uniform(-6, 6, size=(n, 3)).astype(np.float32) - o
    aim = (aim / np.linalg.norm(aim, axis=1, keepdims=True)).astype(np.float32)
    d[::2] = aim[::2]
    return T.make_rays(o, d, 0.0, np.inf)


def tlas_params(max_prims):
    return BvhBuildParams(False, 6, 0, 0.0, 0.0, 0, max_prims, 3.0)


def oracle_scene(blas_tris, tlas_max_prims, blas_params=None):
    blas_params = blas_params or BvhBuildParams.medium_build()
    blas = []
    for t in blas_tris:
        ob = O.build(tris=t, params=blas_params, keep_intermediate=False)
        blas.append((ob.cw_nodes, ob.cw_pidx, t))
    tl = O.build(aabbs=instance_boxes(blas_tris), params=tlas_params(tlas_max_prims), keep_intermediate=False)
    return tl, blas
