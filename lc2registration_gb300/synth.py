"""Seeded synthetic MR/US inputs for the LC2 path.

The reference ships no benchmark data (its YAML files point at private
volumes), so every workload here is synthesised from a seed:

* MR: random ellipses/ellipsoids with intensities U[0,1] on a 0.1
  background, Gaussian blur, plus additive N(0, 0.01^2) noise (std 0.01).
* US: (0.7 MR + 0.5 |Sobel grad MR| + 0.05) resampled through a seeded affine
  onto the US grid, times unit-mean multiplicative Rayleigh speckle
  (numpy ``rayleigh(scale=0.3)`` divided by its mean 0.3*sqrt(pi/2)).

Arrays are float32 in (z, y, x) C order, i.e. x fastest, the reference's
voxel layout (index x + y*X + z*X*Y). The US is the fixed image and the MR the
moving one (the MR is warped into the US grid), i.e. the reference's
``HighResolutionModality: Moving``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from .geometry import Geometry, affine2d, affine3d


def _sobel_mag(img: np.ndarray) -> np.ndarray:
    from scipy import ndimage

    if img.ndim == 2:
        gx = ndimage.correlate(img, np.outer([1, 2, 1], [-1, 0, 1]).astype(np.float64), mode="constant")
        gy = ndimage.correlate(img, np.outer([-1, 0, 1], [1, 2, 1]).astype(np.float64), mode="constant")
        return np.sqrt(gx * gx + gy * gy)
    h = np.array([1.0, 2.0, 1.0])
    hp = np.array([-1.0, 0.0, 1.0])
    k = lambda a, b, c: np.einsum("i,j,k->ijk", a, b, c)  # axes (z, y, x)
    gx = ndimage.correlate(img, k(h, h, hp), mode="constant")
    gy = ndimage.correlate(img, k(h, hp, h), mode="constant")
    gz = ndimage.correlate(img, k(hp, h, h), mode="constant")
    return np.sqrt(gx * gx + gy * gy + gz * gz)


def mr_phantom(shape_zyx: Sequence[int], n_blobs: int, blur_sigma: float, seed: int,
               noise_std: float = 0.01) -> np.ndarray:
    """Random ellipses (2D) or ellipsoids (3D) on a 0.1 background."""
    from scipy import ndimage

    rng = np.random.default_rng(seed)
    shape = tuple(int(s) for s in shape_zyx)
    img = np.full(shape, 0.1, dtype=np.float64)
    nd = len(shape)
    for _ in range(n_blobs):
        c = [rng.uniform(0.2 * s, 0.8 * s) for s in shape]
        ax = [rng.uniform(0.08 * min(shape), 0.25 * min(shape)) for _ in shape]
        val = rng.uniform(0.0, 1.0)
        # evaluate the blob only inside its bounding box
        rad = max(ax)
        lo = [max(0, int(math.floor(cc - rad))) for cc in c]
        hi = [min(s, int(math.ceil(cc + rad)) + 1) for cc, s in zip(c, shape)]
        grids = np.meshgrid(*[np.arange(l, h, dtype=np.float64) for l, h in zip(lo, hi)],
                            indexing="ij")
        box = tuple(slice(l, h) for l, h in zip(lo, hi))
        if nd == 2:
            th = rng.uniform(0, math.pi)
            dy, dx = grids[0] - c[0], grids[1] - c[1]
            u = (dx * math.cos(th) + dy * math.sin(th)) / ax[1]
            v = (-dx * math.sin(th) + dy * math.cos(th)) / ax[0]
            mask = u * u + v * v <= 1.0
        else:
            q = np.linalg.qr(rng.normal(size=(3, 3)))[0]
            d = np.stack([g - cc for g, cc in zip(grids, c)], axis=-1)
            p = d @ q
            mask = ((p / np.array(ax)) ** 2).sum(-1) <= 1.0
        sub = img[box]
        sub[mask] = val
    img = ndimage.gaussian_filter(img, blur_sigma, mode="nearest")
    img += rng.normal(0.0, noise_std, size=shape)
    return img.astype(np.float32)


def _resample_through(src: np.ndarray, src_geom: Geometry, dst_geom: Geometry,
                      mat: np.ndarray) -> np.ndarray:
    """Linear resample of src at dst voxels mapped by mat (dst mm -> src mm)."""
    from scipy import ndimage

    nd = src.ndim
    if nd == 2:
        A = np.asarray(mat, dtype=np.float64).reshape(3, 3)
        ys, xs = np.meshgrid(np.arange(dst_geom.dim[1]), np.arange(dst_geom.dim[0]), indexing="ij")
        lx = xs * dst_geom.spacing[0] + dst_geom.origin[0]
        ly = ys * dst_geom.spacing[1] + dst_geom.origin[1]
        mx = A[0, 0] * lx + A[0, 1] * ly + A[0, 2]
        my = A[1, 0] * lx + A[1, 1] * ly + A[1, 2]
        px = (mx - src_geom.origin[0]) / src_geom.spacing[0]
        py = (my - src_geom.origin[1]) / src_geom.spacing[1]
        return ndimage.map_coordinates(src.astype(np.float64), [py, px], order=1, mode="constant",
                                       cval=0.0)
    A = np.asarray(mat, dtype=np.float64).reshape(4, 4)
    zs, ys, xs = np.meshgrid(np.arange(dst_geom.dim[2]), np.arange(dst_geom.dim[1]),
                             np.arange(dst_geom.dim[0]), indexing="ij")
    l = [xs * dst_geom.spacing[0] + dst_geom.origin[0], ys * dst_geom.spacing[1] + dst_geom.origin[1],
         zs * dst_geom.spacing[2] + dst_geom.origin[2]]
    m = [A[i, 0] * l[0] + A[i, 1] * l[1] + A[i, 2] * l[2] + A[i, 3] for i in range(3)]
    p = [(m[i] - src_geom.origin[i]) / src_geom.spacing[i] for i in range(3)]
    return ndimage.map_coordinates(src.astype(np.float64), [p[2], p[1], p[0]], order=1,
                                   mode="constant", cval=0.0)


def us_from_mr(mr: np.ndarray, mr_geom: Geometry, us_geom: Geometry, mat: np.ndarray,
               seed: int, speckle_scale: float = 0.3) -> np.ndarray:
    """US = (0.7 MR + 0.5 |Sobel MR| + 0.05) o T, times unit-mean Rayleigh speckle."""
    base = 0.7 * mr.astype(np.float64) + 0.5 * _sobel_mag(mr.astype(np.float64)) + 0.05
    us = _resample_through(base, mr_geom, us_geom, mat)
    rng = np.random.default_rng(seed + 7919)
    speck = rng.rayleigh(speckle_scale, size=us.shape) / (speckle_scale * math.sqrt(math.pi / 2))
    return (us * speck).astype(np.float32)


@dataclass
class Case:
    """One synthetic registration problem (what a YAML file describes)."""

    mode: str                      # "2D", "3D" or "2DTo3D"
    fixed_geom: Geometry
    fixed: np.ndarray              # US, float32 (z, y, x)
    moving_geom: Geometry
    moving: np.ndarray             # MR, float32 (z, y, x)
    virt_spacing: List[float]
    r: int
    hr_moving: bool = True
    true_params: dict = field(default_factory=dict)
    true_mat: Optional[np.ndarray] = None

    @property
    def center(self):
        return self.fixed_geom.center()


def case_2d(seed: int = 1, size: int = 256, r: int = 3) -> Case:
    """2D affine: 256x256 MR, 6 ellipses, blur sigma 2 px; US on the same grid
    under rot U[-5,5] deg, trans U[-8,8] px, scale U[0.95,1.05], shear U[-0.03,0.03]."""
    rng = np.random.default_rng(seed)
    mr = mr_phantom((size, size), 6, 2.0, seed)
    g = Geometry((size, size, 1), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0))
    p = dict(rot=rng.uniform(-5, 5), trans=[rng.uniform(-8, 8), rng.uniform(-8, 8)],
             scale=[rng.uniform(0.95, 1.05), rng.uniform(0.95, 1.05)], shear=rng.uniform(-0.03, 0.03))
    c = g.center()[:2]
    mat = affine2d(p["rot"], p["trans"], p["scale"], p["shear"], c, (0.0, 0.0))
    us = us_from_mr(mr, g, g, mat, seed)
    return Case("2D", g, us, g, mr, [1.0, 1.0], r, True, p, mat)


def case_3d(seed: int = 2, mr_size: int = 128, us_size: int = 96, r: int = 3,
            blobs: int = 12, blur: float = 1.5, constant_block_frac: float = 0.0) -> Case:
    """3D affine: MR mr_size^3 at 1 mm, US us_size^3 at 1 mm centred in the MR,
    seeded 12-parameter affine (rot +-8 deg, trans +-10 mm, scale 0.95-1.05,
    shear +-0.03). constant_block_frac > 0 replaces that fraction of the US by
    constant 16^3 blocks (zero-variance patches)."""
    rng = np.random.default_rng(seed)
    mr = mr_phantom((mr_size,) * 3, blobs, blur, seed)
    mg = Geometry((mr_size,) * 3, (1.0, 1.0, 1.0), (0.0, 0.0, 0.0))
    off = (mr_size - us_size) / 2.0
    ug = Geometry((us_size,) * 3, (1.0, 1.0, 1.0), (off, off, off))
    p = dict(rot=list(rng.uniform(-8, 8, 3)), trans=list(rng.uniform(-10, 10, 3)),
             scale=list(rng.uniform(0.95, 1.05, 3)), shear=list(rng.uniform(-0.03, 0.03, 3)))
    mat = affine3d(p["rot"], p["trans"], p["scale"], p["shear"], ug.center(), (0.0, 0.0, 0.0))
    us = us_from_mr(mr, mg, ug, mat, seed)
    if constant_block_frac > 0:
        us = add_constant_blocks(us, constant_block_frac, seed)
    return Case("3D", ug, us, mg, mr, [1.0, 1.0, 1.0], r, True, p, mat)


def add_constant_blocks(us: np.ndarray, frac: float, seed: int, block: int = 16) -> np.ndarray:
    rng = np.random.default_rng(seed + 104729)
    out = us.copy()
    nb = [max(1, s // block) for s in us.shape]
    total = int(np.prod(nb))
    want = int(round(frac * total))
    picks = rng.choice(total, size=want, replace=False)
    for p in picks:
        bz, rem = divmod(int(p), nb[1] * nb[2])
        by, bx = divmod(rem, nb[2])
        sl = (slice(bz * block, (bz + 1) * block), slice(by * block, (by + 1) * block),
              slice(bx * block, (bx + 1) * block))
        out[sl] = np.float32(max(float(out[sl].mean()), 0.05))
    return out


def frame_stack(mr: np.ndarray, mr_geom: Geometry, n_frames: int, seed: int,
                sides=(128, 192, 256, 384, 512), spacing: float = 0.5, r: int = 3) -> List[Case]:
    """2D-to-3D: US frames of uneven square sizes sliced from the MR volume at
    seeded 6-DOF poses (rot +-10 deg, trans +-10 mm) around the MR centre."""
    rng = np.random.default_rng(seed)
    cases = []
    mc = mr_geom.center()
    base = 0.7 * mr.astype(np.float64) + 0.5 * _sobel_mag(mr.astype(np.float64)) + 0.05
    for f in range(n_frames):
        s = int(rng.choice(sides))
        org = (mc[0] - s * spacing / 2, mc[1] - s * spacing / 2, mc[2])
        fg = Geometry((s, s, 1), (spacing, spacing, spacing), org)
        p = dict(rot=list(rng.uniform(-10, 10, 3)), trans=list(rng.uniform(-10, 10, 3)),
                 scale=[1.0, 1.0, 1.0], shear=[0.0, 0.0, 0.0])
        mat = affine3d(p["rot"], p["trans"], p["scale"], p["shear"], fg.center(), (0.0, 0.0, 0.0))
        fr = _resample_through(base, mr_geom, fg, mat).reshape(1, s, s)
        frng = np.random.default_rng(seed * 1000 + f)
        speck = frng.rayleigh(0.3, size=fr.shape) / (0.3 * math.sqrt(math.pi / 2))
        cases.append(Case("2DTo3D", fg, (fr * speck).astype(np.float32), mr_geom, mr,
                          [spacing, spacing, spacing], r, True, p, mat))
    return cases
