"""Shared helpers for the test-suite (scene loading, reference renders)."""
import os

import numpy as np

from obvhs_gb300 import test_util as T
import glam_camera as C

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

#: examples/obj_cwbvh.rs:158 -- normal hash of the 32x18 kitchen render.
KITCHEN_HASH = 1343358762
#: src/cwbvh/traverse_macro.rs:56 -- original id of the hit triangle.
DOCTEST_PRIM = 62


def kitchen_tris():
    z = np.load(os.path.join(GOLDEN, "kitchen_mesh.npz"))
    return z["positions"][z["faces"]].reshape(-1, 9).astype(np.float32)


def kitchen_rays():
    """examples/obj_cwbvh.rs:70-104 at width 32 (height 18)."""
    w = 32
    h = int(np.float32(w) * np.float32(0.5625))
    return C.camera_rays(w, h, C.to_radians(90.0), [3.0, 1.5, 1.4], [-3.9, 1.5, -1.7], [0, 1, 0])


def kitchen_hash(tris, cw_pidx, bvh_ids, rays):
    """Double-sided normals of the hit triangles, hashed like hash_vec3a_vec."""
    hit = bvh_ids != 0xFFFFFFFF
    normals = np.zeros((len(rays), 3), np.float32)
    n = T.compute_normal(tris[cw_pidx[bvh_ids[hit]]])
    dd = T.dot3(n, -rays[hit, 4:7])
    sgn = np.where(np.isnan(dd), dd, np.where(np.signbit(dd), np.float32(-1), np.float32(1))).astype(np.float32)
    normals[hit] = n * sgn[:, None]
    return T.hash_f32_bits(normals)


def doctest_scene():
    """src/cwbvh/traverse_macro.rs:29-33: icosphere(1) + PLANE and one ray."""
    tris = np.concatenate([T.icosphere(1), T.PLANE])
    ray = T.make_rays([[0.1, 0.1, 4.0]], [[0.0, 0.0, -1.0]])
    return tris, ray


def plane_scene():
    """tests/mod.rs:104-124: flat 4x4 plane, 256x256 rays from (0,0.9,0)."""
    tris = T.height_to_triangles(T.flat_heights(4, 4), 4, 4)
    rays = C.camera_rays(256, 256, C.to_radians(90.0), [0, 0.9, 0], [0, 0, 0], [1, 0, 0])
    return tris, rays
