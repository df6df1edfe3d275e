"""Projection and transform builders as float32 arithmetic.

Restates src/Renderer.cpp:40-83 (projectionOrtho, projectionPerspective,
projectionFrustum, projectionFrustumH, projectionCV) and the Matrix4
constructors the samples use (translate, rotateX/Y/Z).  Every operation is a
single numpy float32 scalar operation in the reference's order; tan/sin/cos
are evaluated in double and rounded once.  These build *inputs*: the same
matrix is handed to the device path and to the oracle.
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32


def _m(*vals) -> np.ndarray:
    return np.array(vals, dtype=np.float32).reshape(4, 4)


def projection_ortho(l, r, b, t, n, f) -> np.ndarray:
    l, r, b, t, n, f = map(f32, (l, r, b, t, n, f))
    return _m(f32(2) / (r - l), 0, 0, -(r + l) / (r - l),
              0, f32(2) / (t - b), 0, -(t + b) / (t - b),
              0, 0, f32(-2) / (f - n), -(f + n) / (f - n),
              0, 0, 0, 1)


def projection_perspective(l, r, b, t, n, f) -> np.ndarray:
    l, r, b, t, n, f = map(f32, (l, r, b, t, n, f))
    return _m(f32(2) * n / (r - l), 0, (r + l) / (r - l), 0,
              0, f32(2) * n / (t - b), (t + b) / (t - b), 0,
              0, 0, -(f + n) / (f - n), f32(-2) * f * n / (f - n),
              0, 0, -1, 0)


def tanf(x) -> np.float32:
    return f32(math.tan(float(f32(x))))


def projection_frustum(fov, aspect, n, f) -> np.ndarray:
    fov, aspect, n = f32(fov), f32(aspect), f32(n)
    t = tanf(fov / f32(2))
    return projection_perspective(-n * t * aspect, n * t * aspect, -n * t, n * t, n, f)


def projection_frustum_h(fov, aspect, n, f) -> np.ndarray:
    fov, aspect, n = f32(fov), f32(aspect), f32(n)
    t = tanf(fov / f32(2))
    return projection_perspective(-n * t, n * t, -n * t / aspect, n * t / aspect, n, f)


def projection_ortho_fov(fov, aspect, n, f) -> np.ndarray:
    fov, aspect = f32(fov), f32(aspect)
    return projection_ortho(-fov * aspect / f32(2), fov * aspect / f32(2), -fov / f32(2),
                            fov / f32(2), n, f)


def deg2rad(d) -> np.float32:
    return f32(d) * (f32(3.14159265) / f32(180))


def translate(x, y, z) -> np.ndarray:
    return _m(1, 0, 0, x, 0, 1, 0, y, 0, 0, 1, z, 0, 0, 0, 1)


def scale(s) -> np.ndarray:
    return _m(s, 0, 0, 0, 0, s, 0, 0, 0, 0, s, 0, 0, 0, 0, 1)


def rotate_x(a) -> np.ndarray:
    c, s = f32(math.cos(float(a))), f32(math.sin(float(a)))
    return _m(1, 0, 0, 0, 0, c, -s, 0, 0, s, c, 0, 0, 0, 0, 1)


def rotate_y(a) -> np.ndarray:
    c, s = f32(math.cos(float(a))), f32(math.sin(float(a)))
    return _m(c, 0, s, 0, 0, 1, 0, 0, -s, 0, c, 0, 0, 0, 0, 1)


def rotate_z(a) -> np.ndarray:
    c, s = f32(math.cos(float(a))), f32(math.sin(float(a)))
    return _m(c, -s, 0, 0, s, c, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1)


def mat_mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Row-major 4x4 product, each entry summed left to right in float32."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    r = np.empty((4, 4), np.float32)
    for i in range(4):
        for j in range(4):
            acc = a[i, 0] * b[0, j]
            acc = acc + a[i, 1] * b[1, j]
            acc = acc + a[i, 2] * b[2, j]
            acc = acc + a[i, 3] * b[3, j]
            r[i, j] = acc
    return r


def look_at(eye, target=(0, 0, 0), up=(0, 0, 1)) -> np.ndarray:
    """View matrix for a camera at ``eye`` looking at ``target`` (built in
    double, rounded once)."""
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    upv = np.asarray(up, np.float64)
    if abs(np.dot(fwd, upv)) > 0.99:
        upv = np.array([0.0, 1.0, 0.0])
    right = np.cross(fwd, upv)
    right /= np.linalg.norm(right)
    true_up = np.cross(right, fwd)
    m = np.eye(4)
    m[0, :3] = right
    m[1, :3] = true_up
    m[2, :3] = -fwd
    m[:3, 3] = -m[:3, :3] @ eye
    return m.astype(np.float32)
