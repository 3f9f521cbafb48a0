"""Shared helpers of the parity tests: run one case through the CUDA library
and through the FP64 oracle."""
from __future__ import annotations

import numpy as np

from lc2registration_gb300 import capi
from lc2registration_gb300.geometry import Geometry, affine2d, affine3d
from lc2registration_gb300.synth import Case
from oracle import oracle as O


def round_storage(a: np.ndarray, storage: str) -> np.ndarray:
    """The values the device holds for a given storage type (round to nearest even)."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    if storage == "f32":
        return a
    if storage == "f16":
        return a.astype(np.float16).astype(np.float32)
    bits = a.view(np.uint32).astype(np.uint64)
    lsb = (bits >> 16) & 1
    bits = ((bits + 0x7FFF + lsb) >> 16) << 16
    return bits.astype(np.uint32).view(np.float32)


def ogeom(g: Geometry) -> O.Geom:
    return O.Geom(list(g.dim), list(g.spacing), list(g.origin))


def make_context(case: Case, storage: str = "f32", max_batch: int = 0) -> capi.Context:
    ctx = capi.Context(case.mode, case.fixed_geom, case.moving_geom, case.virt_spacing, case.r,
                       case.hr_moving, storage, max_batch)
    ctx.set_images(case.fixed, case.moving)
    return ctx


def oracle_eval(case: Case, mat, storage: str = "f32", want_fields=False, use_boxsum=True):
    fixed = case.fixed
    moving = round_storage(case.moving, storage)
    if case.hr_moving:
        fixed = round_storage(fixed, storage)
    return O.lc2_eval(case.mode, ogeom(case.fixed_geom), fixed, ogeom(case.moving_geom), moving,
                      case.virt_spacing, case.r, mat, hr_moving=case.hr_moving,
                      use_boxsum=use_boxsum, want_fields=want_fields)


def perturbed(case: Case, rng, n: int, scale: float = 1.0):
    """n matrices around the case's true transform."""
    out = []
    p = case.true_params
    c = case.fixed_geom.center()
    for _ in range(n):
        if case.mode == "2D":
            out.append(affine2d(p["rot"] + scale * rng.uniform(-3, 3),
                                [t + scale * rng.uniform(-4, 4) for t in p["trans"]],
                                [s + scale * rng.uniform(-0.03, 0.03) for s in p["scale"]],
                                p["shear"] + scale * rng.uniform(-0.02, 0.02), c[:2], (0, 0)))
        else:
            out.append(affine3d([a + scale * rng.uniform(-3, 3) for a in p["rot"]],
                                [t + scale * rng.uniform(-4, 4) for t in p["trans"]],
                                [s + scale * rng.uniform(-0.03, 0.03) for s in p["scale"]],
                                [s + scale * rng.uniform(-0.02, 0.02) for s in p["shear"]], c,
                                (0, 0, 0)))
    return np.stack(out)
