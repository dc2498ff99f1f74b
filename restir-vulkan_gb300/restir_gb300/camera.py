"""Pinhole camera in the reference's convention (src/camera.h:25-50).

View rows are (right, -up, forward) with offset -(R * position); the
projection maps view z to clip w, x and y by f/aspect and f, and depth to
[0, 1] between zNear and zFar.  Matrices are produced column-major, as the
reference's uniform buffers hold them.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import _lib


def _dot3(a, b):
    f32 = np.float32
    return f32(f32(f32(a[0] * b[0]) + f32(a[1] * b[1])) + f32(a[2] * b[2]))


def _cross3(a, b):
    f32 = np.float32
    return np.array([f32(a[1] * b[2]) - f32(a[2] * b[1]), f32(a[2] * b[0]) - f32(a[0] * b[2]),
                     f32(a[0] * b[1]) - f32(a[1] * b[0])], f32)


@dataclass
class CameraModel:
    position: np.ndarray
    look_at: np.ndarray
    aspect: float
    fov_y: float = 0.5 * math.pi  # camera.h:16, 90 degrees
    z_near: float = 0.01
    z_far: float = 1000.0
    world_up: tuple = (0.0, 1.0, 0.0)

    def basis(self):
        """Position and unit right, up, forward vectors in float32.  Every
        operation is one IEEE operation on scalars in a fixed order (no BLAS
        dot product, whose order and fused multiply-adds differ between
        machines), so the camera is bit-identical on every host."""
        f32 = np.float32
        pos = np.asarray(self.position, f32)
        fwd = (np.asarray(self.look_at, f32) - pos).astype(f32)
        fwd = (fwd / f32(np.sqrt(_dot3(fwd, fwd)))).astype(f32)
        right = _cross3(fwd, np.asarray(self.world_up, f32))
        right = (right / f32(np.sqrt(_dot3(right, right)))).astype(f32)
        up = _cross3(right, fwd)
        return pos, right, up, fwd

    def view(self) -> np.ndarray:
        pos, right, up, fwd = self.basis()
        rot = np.stack([right, -up, fwd]).astype(np.float64)
        v = np.eye(4)
        v[:3, :3] = rot
        p = pos.astype(np.float64)
        for i in range(3):  # -(rot @ pos), summed left to right
            v[i, 3] = -((rot[i, 0] * p[0] + rot[i, 1] * p[1]) + rot[i, 2] * p[2])
        return v

    def projection(self) -> np.ndarray:
        f = 1.0 / math.tan(0.5 * self.fov_y)
        n, fa = self.z_near, self.z_far
        p = np.zeros((4, 4))
        p[0, 0] = f / self.aspect
        p[1, 1] = f
        p[2, 2] = -fa / (n - fa)
        p[2, 3] = n * fa / (n - fa)
        p[3, 2] = 1.0
        return p

    def projection_view_colmajor(self) -> np.ndarray:
        """P*V as 16 float32 in column-major order (GLSL mat4 memory layout);
        the product is summed left to right in double (no BLAS)."""
        pm, vm = self.projection(), self.view()
        pv = np.zeros((4, 4))
        for i in range(4):
            for j in range(4):
                pv[i, j] = ((pm[i, 0] * vm[0, j] + pm[i, 1] * vm[1, j]) + pm[i, 2] * vm[2, j]) + pm[i, 3] * vm[3, j]
        return pv.astype(np.float32).T.reshape(16).copy()

    def to_c(self) -> _lib.Camera:
        pos, right, up, fwd = self.basis()
        c = _lib.Camera()
        c.position[:] = [float(v) for v in pos]
        c.right[:] = [float(v) for v in right]
        c.up[:] = [float(v) for v in up]
        c.forward[:] = [float(v) for v in fwd]
        c.tan_half_fov_y = float(np.float32(math.tan(0.5 * self.fov_y)))
        c.aspect = float(np.float32(self.aspect))
        c.projection_view[:] = [float(v) for v in self.projection_view_colmajor()]
        return c
