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
        f32 = np.float32
        pos = np.asarray(self.position, f32)
        fwd = np.asarray(self.look_at, f32) - pos
        fwd = (fwd / np.sqrt(np.dot(fwd, fwd))).astype(f32)
        right = np.cross(fwd, np.asarray(self.world_up, f32)).astype(f32)
        right = (right / np.sqrt(np.dot(right, right))).astype(f32)
        up = np.cross(right, fwd).astype(f32)
        return pos, right, up, fwd

    def view(self) -> np.ndarray:
        pos, right, up, fwd = self.basis()
        rot = np.stack([right, -up, fwd]).astype(np.float64)
        off = -(rot @ pos.astype(np.float64))
        v = np.eye(4)
        v[:3, :3] = rot
        v[:3, 3] = off
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
        """P*V as 16 float32 in column-major order (GLSL mat4 memory layout)."""
        return (self.projection() @ self.view()).astype(np.float32).T.reshape(16).copy()

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
