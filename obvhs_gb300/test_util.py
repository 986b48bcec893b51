"""Meshes, generators and sampling helpers mirroring obvhs's `test_util`
module (src/test_util.rs), in numpy float32 with the reference's operation
order (no fused multiply-add, dot products summed as (x+y)+z), plus the
seeded synthetic scenes and ray sets this project benchmarks on.

Triangles are float32 arrays of shape (n, 9): v0 xyz, v1 xyz, v2 xyz.
Rays are float32 arrays of shape (n, 8): origin xyz, tmin, dir xyz, tmax.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import math

import numpy as np

f32 = np.float32

_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
for _name in ("powf", "sinf", "cosf", "sqrtf"):
    getattr(_libm, _name).restype = ctypes.c_float
_libm.powf.argtypes = [ctypes.c_float, ctypes.c_float]
_libm.sinf.argtypes = [ctypes.c_float]
_libm.cosf.argtypes = [ctypes.c_float]
_libm.sqrtf.argtypes = [ctypes.c_float]


def powf(x, y):
    """libm powf, as Rust's f32::powf calls it."""
    return f32(_libm.powf(float(x), float(y)))


def sinf(x):
    return f32(_libm.sinf(float(x)))


def cosf(x):
    return f32(_libm.cosf(float(x)))


# --- sampling (src/test_util.rs:3-126) -------------------------------------

def uhash(x):
    """nullprogram's integer hash (src/test_util.rs:9-17), vectorised, wrapping u32."""
    x = np.asarray(x, dtype=np.uint32)
    with np.errstate(over="ignore"):
        x = x ^ (x >> np.uint32(16))
        x = (x * np.uint32(0x7FEB352D)).astype(np.uint32)
        x = x ^ (x >> np.uint32(15))
        x = (x * np.uint32(0x846CA68B)).astype(np.uint32)
        x = x ^ (x >> np.uint32(16))
    return x


def uhash2(a, b):
    a = np.asarray(a, dtype=np.uint32)
    b = np.asarray(b, dtype=np.uint32)
    with np.errstate(over="ignore"):
        return uhash((a * np.uint32(1597334673)) ^ (b * np.uint32(3812015801)))


def unormf(n):
    return np.asarray(n, dtype=np.uint32).astype(np.float32) * f32(1.0 / 4294967296.0)


def hash_noise(cx, cy, frame):
    with np.errstate(over="ignore"):
        b = (np.asarray(cy, dtype=np.uint32) << np.uint32(11)) + np.uint32(frame)
    return unormf(uhash2(cx, b))


def hash_f32_bits(values) -> int:
    """hash_f32_vec / hash_vec3a_vec (src/test_util.rs:19-30): XOR of uhash of the bit patterns."""
    v = np.ascontiguousarray(values, dtype=np.float32).reshape(-1).view(np.uint32)
    return int(np.bitwise_xor.reduce(uhash(v))) if v.size else 0


def _cubic(v0, v1, v2, v3, x):
    p = (v3 - v2) - (v0 - v1)
    q = (v0 - v1) - p
    r = v2 - v0
    s = v1
    x2 = x * x
    x3 = x2 * x
    return ((p * x3 + q * x2) + r * x) + s


def bicubic_noise(cx, cy, seed):
    """src/test_util.rs:104-126, vectorised over coordinates (float32)."""
    cx = np.asarray(cx, dtype=np.float32)
    cy = np.asarray(cy, dtype=np.float32)
    ix = np.floor(cx).astype(np.int64).clip(0, 0xFFFFFFFF).astype(np.uint32)
    iy = np.floor(cy).astype(np.int64).clip(0, 0xFFFFFFFF).astype(np.uint32)
    fx = cx - ix.astype(np.float32)
    fy = cy - iy.astype(np.float32)

    def col(j):
        with np.errstate(over="ignore"):
            yy = iy + np.uint32(j)
            return _cubic(hash_noise(ix, yy, seed), hash_noise(ix + np.uint32(1), yy, seed),
                          hash_noise(ix + np.uint32(2), yy, seed), hash_noise(ix + np.uint32(3), yy, seed), fx)

    return _cubic(col(0), col(1), col(2), col(3), fy)


def uniform_sample_sphere(u0, u1):
    """src/test_util.rs:73-79 (float32; sin/cos through numpy)."""
    u0 = np.asarray(u0, np.float32)
    u1 = np.asarray(u1, np.float32)
    z = f32(1.0) - f32(2.0) * u0
    r = np.sqrt(f32(1.0) - z * z)
    theta = u1 * f32(2.0 * math.pi)
    return np.stack([r * np.cos(theta), r * np.sin(theta), z], -1).astype(np.float32)


def cosine_sample_hemisphere(u0, u1):
    """src/test_util.rs:62-71."""
    u0 = np.asarray(u0, np.float32)
    u1 = np.asarray(u1, np.float32)
    r = np.sqrt(u0)
    theta = u1 * f32(2.0 * math.pi)
    return np.stack([r * np.cos(theta), r * np.sin(theta), np.sqrt(np.maximum(f32(0.0), f32(1.0) - u0))],
                    -1).astype(np.float32)


def build_orthonormal_basis(n):
    """src/test_util.rs:49-60: returns (x_axis, y_axis, z_axis) columns, each (m, 3)."""
    n = np.asarray(n, np.float32)
    sign = np.where(np.signbit(n[:, 2]), f32(-1.0), f32(1.0)).astype(np.float32)
    a = f32(-1.0) / (sign + n[:, 2])
    b = n[:, 0] * n[:, 1] * a
    x_axis = np.stack([f32(1.0) + sign * n[:, 0] * n[:, 0] * a, sign * b, -sign * n[:, 0]], -1)
    y_axis = np.stack([b, sign + n[:, 1] * n[:, 1] * a, -n[:, 1]], -1)
    return x_axis.astype(np.float32), y_axis.astype(np.float32), n


# --- vector helpers with glam's Vec3A operation order -----------------------

def dot3(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def cross3(a, b):
    return np.stack([a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1], a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
                     a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0]], -1)


def normalize3(v):
    """glam Vec3A::normalize: v * (1 / sqrt(dot(v, v)))."""
    v = np.asarray(v, np.float32)
    rcp = f32(1.0) / np.sqrt(dot3(v, v))
    return v * rcp[..., None]


def normalize_or_zero3(v):
    v = np.asarray(v, np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        rcp = f32(1.0) / np.sqrt(dot3(v, v))
    ok = np.isfinite(rcp) & (rcp > 0)
    out = v * np.where(ok, rcp, f32(0.0))[..., None]
    return np.where(ok[..., None], out, f32(0.0)).astype(np.float32)


def compute_normal(tris):
    """Triangle::compute_normal (src/triangle.rs:18-24)."""
    t = np.asarray(tris, np.float32).reshape(-1, 3, 3)
    e1 = t[:, 1] - t[:, 0]
    e2 = t[:, 2] - t[:, 0]
    return normalize_or_zero3(cross3(e1, e2))


# --- geometry (src/test_util.rs:170-305) ------------------------------------

def _tri(a, b, c):
    return [*a, *b, *c]


CUBE = np.array([
    _tri((-1., 1., -1.), (1., 1., 1.), (1., 1., -1.)),
    _tri((1., 1., 1.), (-1., -1., 1.), (1., -1., 1.)),
    _tri((-1., 1., 1.), (-1., -1., -1.), (-1., -1., 1.)),
    _tri((1., -1., -1.), (-1., -1., 1.), (-1., -1., -1.)),
    _tri((1., 1., -1.), (1., -1., 1.), (1., -1., -1.)),
    _tri((-1., 1., -1.), (1., -1., -1.), (-1., -1., -1.)),
    _tri((-1., 1., -1.), (-1., 1., 1.), (1., 1., 1.)),
    _tri((1., 1., 1.), (-1., 1., 1.), (-1., -1., 1.)),
    _tri((-1., 1., 1.), (-1., 1., -1.), (-1., -1., -1.)),
    _tri((1., -1., -1.), (1., -1., 1.), (-1., -1., 1.)),
    _tri((1., 1., -1.), (1., 1., 1.), (1., -1., 1.)),
    _tri((-1., 1., -1.), (1., 1., -1.), (1., -1., -1.)),
], np.float32)

PLANE = np.array([
    _tri((1., 0., 1.), (-1., 0., -1.), (-1., 0., 1.)),
    _tri((1., 0., 1.), (1., 0., -1.), (-1., 0., -1.)),
], np.float32)


def icosphere(subdivisions: int) -> np.ndarray:
    """src/test_util.rs:205-252."""
    phi = (f32(1.0) + np.sqrt(f32(5.0))) / f32(2.0)
    a, b, c, d, e = f32(1.0), f32(-1.0), f32(0.0), phi, -phi
    p = np.array([(b, d, c), (a, d, c), (b, e, c), (a, e, c), (c, b, d), (c, a, d), (c, b, e), (c, a, e), (d, c, b),
                  (d, c, a), (e, c, b), (e, c, a)], np.float32)
    p = normalize3(p)
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    tris = np.array([[p[i], p[j], p[k]] for i, j, k in faces], np.float32)  # (20, 3, 3)
    for _ in range(subdivisions):
        v0, v1, v2 = tris[:, 0], tris[:, 1], tris[:, 2]
        m01 = normalize3((v0 + v1) * f32(0.5))
        m12 = normalize3((v1 + v2) * f32(0.5))
        m20 = normalize3((v2 + v0) * f32(0.5))
        new = np.stack([np.stack([v0, m01, m20], 1), np.stack([v1, m12, m01], 1), np.stack([v2, m20, m12], 1),
                        np.stack([m01, m12, m20], 1)], 1)  # (t, 4, 3, 3)
        tris = new.reshape(-1, 3, 3)
    return tris.reshape(-1, 9).astype(np.float32)


def height_to_triangles(heights: np.ndarray, x_res: int, z_res: int) -> np.ndarray:
    """src/test_util.rs:254-287.  heights[x, z] holds height_map(x, z) on the
    (x_res+1) x (z_res+1) grid."""
    xr = f32(x_res)
    zr = f32(z_res)
    out = np.empty((z_res, x_res, 2, 9), np.float32)
    xs = np.arange(x_res + 1, dtype=np.float32)
    zs = np.arange(z_res + 1, dtype=np.float32)
    fxs = (xs / xr) * f32(2.0) - f32(1.0)
    fzs = (zs / zr) * f32(2.0) - f32(1.0)
    for z in range(z_res):
        fx, fx2 = fxs[:-1], fxs[1:]
        fz, fz2 = fzs[z], fzs[z + 1]
        h00 = heights[:-1, z]
        h10 = heights[1:, z]
        h01 = heights[:-1, z + 1]
        h11 = heights[1:, z + 1]
        fzv = np.full(x_res, fz, np.float32)
        fz2v = np.full(x_res, fz2, np.float32)
        v00 = np.stack([fx, h00, fzv], -1)
        v10 = np.stack([fx2, h10, fzv], -1)
        v01 = np.stack([fx, h01, fz2v], -1)
        v11 = np.stack([fx2, h11, fz2v], -1)
        out[z, :, 0] = np.concatenate([v00, v01, v10], -1)
        out[z, :, 1] = np.concatenate([v10, v01, v11], -1)
    return out.reshape(-1, 9)


def flat_heights(x_res: int, z_res: int) -> np.ndarray:
    return np.zeros((x_res + 1, z_res + 1), np.float32)


def demoscene(terrain_res: int, seed: int) -> np.ndarray:
    """src/test_util.rs:289-304 (float32; powf through libm)."""
    n = terrain_res + 1
    xs, ys = np.meshgrid(np.arange(n, dtype=np.float32), np.arange(n, dtype=np.float32), indexing="ij")
    res = f32(terrain_res)
    cx = xs / res
    cy = ys / res
    cs, ns = f32(1.579), f32(0.579)
    acc = np.zeros_like(cx)
    for i in range(1, 17):
        cs, ns = f32(cs * f32(1.579)), f32(ns * f32(-0.579))
        acc = acc + bicubic_noise(cx * cs, cy * cs, seed + i) * ns
    one_m = f32(1.0) - cy[0]
    p1 = np.array([powf(v, 0.579) for v in one_m], np.float32)
    p2 = np.array([powf(v, 1.579) for v in one_m], np.float32)
    heights = acc * p1[None, :] + p2[None, :] * f32(0.579)
    return height_to_triangles(heights.astype(np.float32), terrain_res, terrain_res)


def tri_aabbs(tris: np.ndarray) -> np.ndarray:
    """Triangle::aabb with SSE min/max lane semantics (a<b?a:b)."""
    t = np.asarray(tris, np.float32).reshape(-1, 3, 3)

    def smin(a, b):
        return np.where(a < b, a, b)

    def smax(a, b):
        return np.where(a > b, a, b)

    mn = smin(smin(t[:, 0], t[:, 1]), t[:, 2])
    mx = smax(smax(t[:, 0], t[:, 1]), t[:, 2])
    return np.concatenate([mn, mx], -1).astype(np.float32)


def make_rays(origins, dirs, tmin=0.0, tmax=np.inf) -> np.ndarray:
    o = np.asarray(origins, np.float32).reshape(-1, 3)
    d = np.asarray(dirs, np.float32).reshape(-1, 3)
    n = max(len(o), len(d))
    r = np.empty((n, 8), np.float32)
    r[:, 0:3] = o
    r[:, 3] = np.broadcast_to(np.asarray(tmin, np.float32), (n,))
    r[:, 4:7] = d
    r[:, 7] = np.broadcast_to(np.asarray(tmax, np.float32), (n,))
    return r
