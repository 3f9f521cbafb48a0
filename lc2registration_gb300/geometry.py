"""Image geometry and the reference's transform builders (host side, FP64).

Restates the reference's mapper math:

* ``Geometry.center`` -- PhysioSpatial{2,3}DMapper centre
  ``origin + spacing * dim / 2`` (src/Interpolator/spatialMappers.cuh:59-65).
* ``virtual_geometry`` -- the virtual grid: fixed origin, dims
  ``ceil(dimF * spF / spV)`` (src/Interpolator/interpolator.cu:337-339).
* ``affine3d`` -- Spatial3DMapper::AffineInit (spatialMappers.cuh:637-850):
  ``x_m = L (x_v - C + shift) + C + T`` with ``L = Rz Ry Rx Sh S``,
  ``Sh = [[1, shx, shy], [0, 1, shz], [0, 0, 1]]``, angles in degrees.
* ``affine2d`` -- Spatial2DMapper::AffineInit (spatialMappers.cuh:999-1033),
  ``L = R Sh S`` with ``Sh = [[1, sh], [0, 1]]``.
* ``moving_to_fixed`` -- GetMovingToFixedTransform: VirtualToFixed (identity)
  times the inverse of VirtualToMoving (src/Interpolator/interpolator.cu:651-679).

The matrices are built in double and rounded once to float32 (the reference
builds them in float32 from double sin/cos); the C library's builders
(``lc2_affine3d``/``lc2_affine2d``) use the same formulas.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Sequence, Tuple

import numpy as np


@dataclass
class Geometry:
    dim: Tuple[int, int, int]
    spacing: Tuple[float, float, float]
    origin: Tuple[float, float, float]

    def __post_init__(self):
        d = list(self.dim) + [1] * (3 - len(self.dim))
        s = list(self.spacing) + [1.0] * (3 - len(self.spacing))
        o = list(self.origin) + [0.0] * (3 - len(self.origin))
        self.dim = tuple(int(v) for v in d[:3])
        self.spacing = tuple(float(np.float32(v)) for v in s[:3])
        self.origin = tuple(float(np.float32(v)) for v in o[:3])

    @property
    def n(self) -> int:
        return int(self.dim[0] * self.dim[1] * self.dim[2])

    @property
    def shape_zyx(self):
        return (self.dim[2], self.dim[1], self.dim[0])

    def center(self) -> Tuple[float, float, float]:
        """Physical centre, float32 arithmetic as in the reference mapper."""
        f = np.float32
        return tuple(float(f(self.origin[a]) + f(self.spacing[a]) * f(self.dim[a]) / f(2.0))
                     for a in range(3))


def virtual_geometry(ndim: int, fixed: Geometry, virt_spacing: Sequence[float]) -> Geometry:
    f = np.float32
    sv = list(virt_spacing) + [1.0] * (3 - len(virt_spacing))
    dims = []
    for a in range(3):
        if a < ndim:
            dims.append(int(math.ceil(float(f(f(fixed.dim[a]) * f(fixed.spacing[a])) / f(sv[a])))))
        else:
            dims.append(1)
    sp = [sv[0], sv[1], sv[2] if ndim == 3 else 1.0]
    org = [fixed.origin[0], fixed.origin[1], fixed.origin[2] if ndim == 3 else 0.0]
    return Geometry(tuple(dims), tuple(sp), tuple(org))


def _rot3(rx, ry, rz):
    d = math.pi / 180.0
    cx, sx = math.cos(rx * d), math.sin(rx * d)
    cy, sy = math.cos(ry * d), math.sin(ry * d)
    cz, sz = math.cos(rz * d), math.sin(rz * d)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def affine3d(rot, trans, scale=(1, 1, 1), shear=(0, 0, 0), center=(0, 0, 0),
             shift=(0, 0, 0)) -> np.ndarray:
    """Row-major float32 4x4 virtual->moving matrix."""
    Sh = np.array([[1.0, shear[0], shear[1]], [0.0, 1.0, shear[2]], [0.0, 0.0, 1.0]])
    S = np.diag([float(v) for v in scale])
    L = _rot3(*[float(v) for v in rot]) @ Sh @ S
    C = np.array(center, dtype=np.float64)
    t = L @ (np.array(shift, dtype=np.float64) - C) + C + np.array(trans, dtype=np.float64)
    M = np.eye(4)
    M[:3, :3] = L
    M[:3, 3] = t
    return M.astype(np.float32)


def affine2d(rot, trans, scale=(1, 1), shear=0.0, center=(0, 0), shift=(0, 0)) -> np.ndarray:
    """Row-major float32 3x3 virtual->moving matrix."""
    d = math.pi / 180.0
    c, s = math.cos(float(rot) * d), math.sin(float(rot) * d)
    L = np.array([[c, -s], [s, c]]) @ np.array([[1.0, float(shear)], [0.0, 1.0]]) @ np.diag(
        [float(scale[0]), float(scale[1])])
    C = np.array(center[:2], dtype=np.float64)
    t = L @ (np.array(shift[:2], dtype=np.float64) - C) + C + np.array(trans[:2], dtype=np.float64)
    M = np.eye(3)
    M[:2, :2] = L
    M[:2, 2] = t
    return M.astype(np.float32)


def params_to_matrix(mode: str, params: Sequence[float], center, shift) -> np.ndarray:
    """Parameter vector in the reference's order -> matrix.

    2D: [TX, TY, R, ScaleX, ScaleY, Shear] (src/Optimizers/optimizers.cu:30-36);
    3D and 2DTo3D: [TX, TY, TZ, RX, RY, RZ, ScaleX..Z, ShearX..Z]
    (optimizers.cu:497-509).
    """
    p = [float(v) for v in params]
    if mode == "2D":
        return affine2d(p[2], p[0:2], p[3:5], p[5], center, shift)
    return affine3d(p[3:6], p[0:3], p[6:9], p[9:12], center, shift)


def moving_to_fixed(mat: np.ndarray) -> np.ndarray:
    """VirtualToFixed (identity) x inverse(VirtualToMoving)."""
    return np.linalg.inv(np.asarray(mat, dtype=np.float64)).astype(np.float32)
