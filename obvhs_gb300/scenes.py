"""Seeded synthetic scenes and ray sets for the benchmark workloads.

No public dataset is involved; every array comes from numpy's PCG64 seeded
with 1000 + the workload number (+ a per-scene offset).
  scene 1: 10,000 triangles, centroids U[-1,1]^3, vertices = centroid +
           U[-0.02,0.02]^3; 256x256 pinhole rays from (0,0,-3) along +z,
           60 deg vertical field of view, pixel centres, tmin 0, tmax inf.
  scene 2: 1M triangles in 64 Gaussian clusters (centres U[-10,10]^3, sigma
           log-uniform [0.1,2]), equilateral triangles with log-normal edge
           (mu ln 0.01, sigma 0.7) in random orientation; 1920x1080 primary
           rays from a pinhole framing the densest cluster (scene2_camera),
           then one cosine-weighted bounce per primary hit.
  scene 3: 8M triangles: 40% from 200 axis-aligned quads tessellated into
           triangles of 0.05-0.5, 60% clutter (edge 0.002-0.02) in a 20x6x20
           box; 16M rays with uniform origins in the box and uniform sphere
           directions, plus 16M shadow rays to 4 point lights.
"""
from __future__ import annotations

import math

import numpy as np

from . import test_util as T

f32 = np.float32


def _rng(workload: int, offset: int = 0):
    return np.random.Generator(np.random.PCG64(1000 + workload + offset))


def pinhole_rays(width: int, height: int, origin, vfov_deg: float = 60.0, tmax=np.inf):
    """Pixel-centre rays of a pinhole camera looking along +z (y up)."""
    th = f32(math.tan(math.radians(vfov_deg) / 2))
    aspect = f32(width) / f32(height)
    xs = (np.arange(width, dtype=np.float32) + f32(0.5)) / f32(width) * f32(2) - f32(1)
    ys = f32(1) - (np.arange(height, dtype=np.float32) + f32(0.5)) / f32(height) * f32(2)
    gx, gy = np.meshgrid(xs * th * aspect, ys * th)
    d = np.stack([gx.ravel(), gy.ravel(), np.ones(width * height, np.float32)], -1)
    d = T.normalize3(d)
    return T.make_rays(np.broadcast_to(np.asarray(origin, np.float32), d.shape), d, 0.0, tmax)


def scene1(n: int = 10_000):
    rng = _rng(1)
    c = rng.uniform(-1, 1, size=(n, 1, 3))
    v = c + rng.uniform(-0.02, 0.02, size=(n, 3, 3))
    tris = v.reshape(n, 9).astype(np.float32)
    return tris, pinhole_rays(256, 256, (0.0, 0.0, -3.0))


def _equilateral(rng, centres, edge):
    n = len(centres)
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    tmp = rng.normal(size=(n, 3))
    t = tmp - (tmp * nrm).sum(1, keepdims=True) * nrm
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    b = np.cross(nrm, t)
    phi = rng.uniform(0, 2 * np.pi, size=(n, 1))
    r = (edge / np.sqrt(3.0))[:, None]
    verts = []
    for k in range(3):
        a = phi + 2 * np.pi * k / 3
        verts.append(centres + r * (np.cos(a) * t + np.sin(a) * b))
    return np.concatenate(verts, 1).astype(np.float32)


def _scene2_clusters(rng, clusters: int):
    centres = rng.uniform(-10, 10, size=(clusters, 3))
    sigma = np.exp(rng.uniform(np.log(0.1), np.log(2.0), size=clusters))
    return centres, sigma


def scene2_tris(n: int = 1_000_000, clusters: int = 64, offset: int = 0):
    rng = _rng(2, offset)
    centres, sigma = _scene2_clusters(rng, clusters)
    which = rng.integers(0, clusters, size=n)
    cen = centres[which] + rng.normal(size=(n, 3)) * sigma[which, None]
    edge = rng.lognormal(np.log(0.01), 0.7, size=n)
    return _equilateral(rng, cen, edge)


#: camera distance from the framed cluster's centre, in that cluster's sigma
SCENE2_CAMERA_SIGMAS = 3.0


def scene2_camera(clusters: int = 64, offset: int = 0):
    """Pinhole origin for the scene-2 primary rays: SCENE2_CAMERA_SIGMAS
    sigmas in front (-z) of the densest cluster (smallest sigma), looking
    along +z at its centre.  The clusters are optically thin from far away
    (a camera framing the whole [-10,10]^3 box sees ~2% of its pixels hit),
    so the camera frames one cluster that fills the view: ~85% of the
    1920x1080 rays hit, and each hit spawns a bounce ray."""
    centres, sigma = _scene2_clusters(_rng(2, offset), clusters)
    k = int(np.argmin(sigma))
    o = centres[k] - np.array([0.0, 0.0, SCENE2_CAMERA_SIGMAS * sigma[k]])
    return tuple(float(x) for x in o.astype(np.float32))


def scene2_primary_rays(width: int = 1920, height: int = 1080):
    return pinhole_rays(width, height, scene2_camera(), 60.0)


def bounce_rays(tris, rays, prim_ids, t, seed: int = 2):
    """One cosine-weighted diffuse bounce per hit (test_util.rs:49-71;
    origin = hit point - 0.01 * direction as in examples/demoscene.rs:169)."""
    hit = prim_ids != 0xFFFFFFFF
    if not hit.any():
        return np.zeros((0, 8), np.float32)
    r = rays[hit]
    d = r[:, 4:7]
    o = r[:, 0:3]
    tt = t[hit][:, None]
    n = T.compute_normal(tris[prim_ids[hit]])
    dd = T.dot3(n, -d)
    n = n * np.where(np.signbit(dd), f32(-1), f32(1))[:, None]
    p = o + d * tt - d * f32(0.01)
    rng = _rng(seed, 7)
    u = rng.random(size=(len(r), 2)).astype(np.float32)
    local = T.cosine_sample_hemisphere(u[:, 0], u[:, 1])
    x_axis, y_axis, z_axis = T.build_orthonormal_basis(n)
    w = x_axis * local[:, 0:1] + y_axis * local[:, 1:2] + z_axis * local[:, 2:3]
    w = T.normalize3(w)
    return T.make_rays(p, w, 0.0, np.inf)


def scene3_tris(n: int = 8_000_000, offset: int = 0):
    rng = _rng(3, offset)
    n_wall = int(n * 0.4)
    n_clutter = n - n_wall
    # 200 axis-aligned quads tessellated into right-triangle pairs
    quads = 200
    per = n_wall // quads
    out = []
    for q in range(quads):
        cnt = per if q < quads - 1 else n_wall - per * (quads - 1)
        cells = max(1, cnt // 2)
        axis = rng.integers(0, 3)
        size = rng.uniform(0.05, 0.5)
        side = int(math.ceil(math.sqrt(cells)))
        origin = rng.uniform([-10, -3, -10], [10, 3, 10])
        ij = np.arange(cells)
        i = (ij % side).astype(np.float64)
        j = (ij // side).astype(np.float64)
        u_axis, v_axis = [(1, 2), (0, 2), (0, 1)][axis]
        base = np.zeros((cells, 3))
        base[:] = origin
        base[:, u_axis] += i * size
        base[:, v_axis] += j * size
        du = np.zeros(3)
        du[u_axis] = size
        dv = np.zeros(3)
        dv[v_axis] = size
        a, b, c, d = base, base + du, base + du + dv, base + dv
        t1 = np.concatenate([a, b, c], 1)
        t2 = np.concatenate([a, c, d], 1)
        tri = np.stack([t1, t2], 1).reshape(-1, 9)[:cnt]
        if len(tri) < cnt:
            tri = np.concatenate([tri, tri[: cnt - len(tri)]])
        out.append(tri)
    walls = np.concatenate(out).astype(np.float32)
    cen = rng.uniform([-10, -3, -10], [10, 3, 10], size=(n_clutter, 3))
    edge = rng.uniform(0.002, 0.02, size=n_clutter)
    clutter = _equilateral(rng, cen, edge)
    tris = np.concatenate([walls, clutter])
    return tris[rng.permutation(len(tris))]


def scene3_rays(n: int = 16_000_000, lights: int = 4, offset: int = 0):
    rng = _rng(3, 100 + offset)
    o = rng.uniform([-10, -3, -10], [10, 3, 10], size=(n, 3)).astype(np.float32)
    u = rng.random(size=(n, 2)).astype(np.float32)
    d = T.uniform_sample_sphere(u[:, 0], u[:, 1])
    closest = T.make_rays(o, d, 0.0, np.inf)
    lp = rng.uniform([-9, 2, -9], [9, 2.9, 9], size=(lights, 3)).astype(np.float32)
    which = rng.integers(0, lights, size=n)
    to = lp[which] - o
    dist = np.sqrt((to.astype(np.float64) ** 2).sum(1))
    sd = (to / dist[:, None]).astype(np.float32)
    shadow = T.make_rays(o, sd, 0.0, (dist * (1 - 1e-4)).astype(np.float32))
    return closest, shadow
