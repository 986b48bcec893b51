"""Camera rays exactly as the reference's tests and examples make them.

Restates, in numpy float32, the glam (0.30) matrix helpers that
tests/mod.rs:151-169 and examples/obj_cwbvh.rs:70-104 use:
Mat4::perspective_infinite_reverse_rh, Mat4::look_at_rh, Mat4::inverse
(GLM's cofactor form, as in glam's scalar backend), Mat4 * Vec4, and
Vec3A::normalize.  glam itself is a third-party crate that is not in the
reference tree; these are restatements of its published algorithms.
Matrices are column-major: m[c] is column c.
"""
from __future__ import annotations

import ctypes
import ctypes.util

import numpy as np

f32 = np.float32
_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.sinf.restype = ctypes.c_float
_libm.cosf.restype = ctypes.c_float
_libm.sinf.argtypes = [ctypes.c_float]
_libm.cosf.argtypes = [ctypes.c_float]


def to_radians(deg: float) -> np.float32:
    """f32::to_radians: deg * (PI / 180) with the constant folded in f32."""
    return f32(f32(deg) * f32(f32(np.pi) / f32(180.0)))


def perspective_infinite_reverse_rh(fov_y, aspect, z_near):
    half = f32(f32(0.5) * f32(fov_y))
    s = f32(_libm.sinf(float(half)))
    c = f32(_libm.cosf(float(half)))
    h = f32(c / s)
    w = f32(h / f32(aspect))
    m = np.zeros((4, 4), np.float32)
    m[0] = [w, 0, 0, 0]
    m[1] = [0, h, 0, 0]
    m[2] = [0, 0, 0, -1]
    m[3] = [0, 0, f32(z_near), 0]
    return m


def _dot3(a, b):
    return f32(f32(f32(a[0] * b[0]) + f32(a[1] * b[1])) + f32(a[2] * b[2]))


def _norm3(v):
    v = np.asarray(v, np.float32)
    rcp = f32(f32(1.0) / np.sqrt(_dot3(v, v)))
    return (v * rcp).astype(np.float32)


def _cross3(a, b):
    return np.array([a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1]], np.float32)


def look_at_rh(eye, center, up):
    eye = np.asarray(eye, np.float32)
    f = _norm3(np.asarray(center, np.float32) - eye)
    s = _norm3(_cross3(f, np.asarray(up, np.float32)))
    u = _cross3(s, f)
    m = np.zeros((4, 4), np.float32)
    m[0] = [s[0], u[0], -f[0], 0]
    m[1] = [s[1], u[1], -f[1], 0]
    m[2] = [s[2], u[2], -f[2], 0]
    m[3] = [-_dot3(eye, s), -_dot3(eye, u), _dot3(eye, f), 1]
    return m


def inverse(m):
    """glam Mat4::inverse (GLM cofactor expansion), float32 step by step."""
    m = np.asarray(m, np.float32)
    (m00, m01, m02, m03), (m10, m11, m12, m13), (m20, m21, m22, m23), (m30, m31, m32, m33) = m

    def d(a, b, c, e):
        return f32(f32(a * b) - f32(c * e))

    coef00 = d(m22, m33, m32, m23)
    coef02 = d(m12, m33, m32, m13)
    coef03 = d(m12, m23, m22, m13)
    coef04 = d(m21, m33, m31, m23)
    coef06 = d(m11, m33, m31, m13)
    coef07 = d(m11, m23, m21, m13)
    coef08 = d(m21, m32, m31, m22)
    coef10 = d(m11, m32, m31, m12)
    coef11 = d(m11, m22, m21, m12)
    coef12 = d(m20, m33, m30, m23)
    coef14 = d(m10, m33, m30, m13)
    coef15 = d(m10, m23, m20, m13)
    coef16 = d(m20, m32, m30, m22)
    coef18 = d(m10, m32, m30, m12)
    coef19 = d(m10, m22, m20, m12)
    coef20 = d(m20, m31, m30, m21)
    coef22 = d(m10, m31, m30, m11)
    coef23 = d(m10, m21, m20, m11)
    V = lambda *a: np.array(a, np.float32)  # noqa: E731
    fac0 = V(coef00, coef00, coef02, coef03)
    fac1 = V(coef04, coef04, coef06, coef07)
    fac2 = V(coef08, coef08, coef10, coef11)
    fac3 = V(coef12, coef12, coef14, coef15)
    fac4 = V(coef16, coef16, coef18, coef19)
    fac5 = V(coef20, coef20, coef22, coef23)
    vec0 = V(m10, m00, m00, m00)
    vec1 = V(m11, m01, m01, m01)
    vec2 = V(m12, m02, m02, m02)
    vec3 = V(m13, m03, m03, m03)
    inv0 = (vec1 * fac0 - vec2 * fac1) + vec3 * fac2
    inv1 = (vec0 * fac0 - vec2 * fac3) + vec3 * fac4
    inv2 = (vec0 * fac1 - vec1 * fac3) + vec3 * fac5
    inv3 = (vec0 * fac2 - vec1 * fac4) + vec2 * fac5
    sign_a = V(1, -1, 1, -1)
    sign_b = V(-1, 1, -1, 1)
    inv = np.stack([inv0 * sign_a, inv1 * sign_b, inv2 * sign_a, inv3 * sign_b]).astype(np.float32)
    col0 = V(inv[0][0], inv[1][0], inv[2][0], inv[3][0])
    dot0 = m[0] * col0
    dot1 = f32(f32(f32(dot0[0] + dot0[1]) + dot0[2]) + dot0[3])
    rcp = f32(f32(1.0) / dot1)
    return (inv * rcp).astype(np.float32)


def mat_vec(m, v):
    """Mat4 * Vec4: ((x_axis*v.x + y_axis*v.y) + z_axis*v.z) + w_axis*v.w, per lane."""
    m = np.asarray(m, np.float32)
    v = np.asarray(v, np.float32)  # (..., 4)
    r = m[0] * v[..., 0:1]
    r = r + m[1] * v[..., 1:2]
    r = r + m[2] * v[..., 2:3]
    r = r + m[3] * v[..., 3:4]
    return r.astype(np.float32)


def camera_rays(width, height, fov_y, eye, look_at, up, tmax=np.float32(3.4028235e38)):
    """Rays in frag order i = y*width + x (src of obj_cwbvh.rs:94-104)."""
    tsx, tsy = f32(width), f32(height)
    aspect = f32(tsx / tsy)
    proj_inv = inverse(perspective_infinite_reverse_rh(fov_y, aspect, f32(0.01)))
    view_inv = inverse(look_at_rh(eye, look_at, up))
    i = np.arange(width * height)
    fx = (i % width).astype(np.float32)
    fy = (i // width).astype(np.float32)
    ux = fx / tsx
    uy = f32(1.0) - fy / tsy
    nx = ux * f32(2.0) - f32(1.0)
    ny = uy * f32(2.0) - f32(1.0)
    clip = np.stack([nx, ny, np.ones_like(nx), np.ones_like(nx)], -1).astype(np.float32)
    vs = mat_vec(proj_inv, clip)
    vs = (vs / vs[:, 3:4]).astype(np.float32)
    world = mat_vec(view_inv, vs)[:, :3]
    d = world - np.asarray(eye, np.float32)
    dd = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    d = (d * (f32(1.0) / np.sqrt(dd))[:, None]).astype(np.float32)
    rays = np.empty((len(i), 8), np.float32)
    rays[:, 0:3] = np.asarray(eye, np.float32)
    rays[:, 3] = 0.0
    rays[:, 4:7] = d
    rays[:, 7] = tmax
    return rays
