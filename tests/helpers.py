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


def write_param_file(tmp_path, case, name="params.yaml", direct=True, rounds=None,
                     centred=False, patch=None):
    """Writes a parameter file in the reference's schema (config/*.yaml) for a
    synthetic case, with the images as raw float32 files next to it."""
    nd = 2 if case.mode == "2D" else 3
    f, m = tmp_path / "fixed.raw", tmp_path / "moving.raw"
    case.fixed.astype(np.float32).tofile(f)
    case.moving.astype(np.float32).tofile(m)
    ax = ["x", "y", "z"][:nd]

    def geo(g):
        d = ", ".join(f"{a}: {int(g.dim[i])}" for i, a in enumerate(ax))
        s = ", ".join(f"{a}: {g.spacing[i]!r}" for i, a in enumerate(ax))
        o = ", ".join(f"{a}: {g.origin[i]!r}" for i, a in enumerate(ax))
        return f"{{{d}}}", f"{{{s}}}", f"{{{o}}}"

    fd, fs, fo = geo(case.fixed_geom)
    md, ms, mo = geo(case.moving_geom)
    img = "Image" if nd == 2 else "Volume"
    vs = ", ".join(f"{a}: {case.virt_spacing[i]!r}" for i, a in enumerate(ax))
    if nd == 2:
        keys = ["TX", "TY", "R", "ScaleX", "ScaleY", "Shear"]
        init = [0, 0, 0, 1, 1, 0]
        lo = [-10, -10, -8, 0.9, 0.9, -0.06]
        hi = [10, 10, 8, 1.1, 1.1, 0.06]
    else:
        keys = ["TX", "TY", "TZ", "RX", "RY", "RZ", "ScaleX", "ScaleY", "ScaleZ", "ShearX",
                "ShearY", "ShearZ"]
        init = [0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0]
        lo = [-10, -10, -10, -8, -8, -8, 0.9, 0.9, 0.9, -0.05, -0.05, -0.05]
        hi = [10, 10, 10, 8, 8, 8, 1.1, 1.1, 1.1, 0.05, 0.05, 0.05]
    kv = lambda vals: "{" + ", ".join(f"{k}: {float(v)!r}" for k, v in zip(keys, vals)) + "}"
    rounds = rounds or [("true", "true", "false", "false", "1.0e-4"),
                        ("true", "true", "true", "true", "1.0e-4")]
    lines = [
        "InputParameters:",
        f"  Fixed{img}:",
        f"    Dimension: {fd}",
        f"    Spacing: {fs}",
        f"    Origin: {fo}",
        f"    FilePath: {f}",
        "    Format: raw",
        "    DataType: float32",
        f"  Moving{img}:",
        f"    Dimension: {md}",
        f"    Spacing: {ms}",
        f"    Origin: {mo}",
        f"    FilePath: {m}  # raw float32",
        "    Format: raw",
        "  RegistrationParameters:",
        f"    HighResolutionModality: {'Moving' if case.hr_moving else 'Fixed'}",
        "    Type: Affine",
        f"    ResampledSpacing: {{{vs}}}",
        f"    PatchSize: {patch or case.r}",
        f"    FinalRoundExportRootPath: {tmp_path}",
        f"    CenterOverlaid: {'true' if centred else 'false'}",
        "  OptimizerSettings:",
        f"    InitialValues: {kv(init)}",
        f"    LowerBounds: {kv([l - i if k in ('TX', 'TY', 'TZ', 'R', 'RX', 'RY', 'RZ') else l for k, l, i in zip(keys, lo, init)])}",
        f"    UpperBounds: {kv([h - i if k in ('TX', 'TY', 'TZ', 'R', 'RX', 'RY', 'RZ') else h for k, h, i in zip(keys, hi, init)])}",
        "    DIRECT:",
        f"      Enabled: {'true' if direct else 'false'}",
        "      OptimizedEntries: {Translation: true, Rotation: false, Scale: false, Shear: false}",
        "      MaxEvaluations: 50",
        "    BOBYQA:",
    ]
    for r, (t, ro, s, sh, tol) in enumerate(rounds):
        lines += [f"      {r}:", "        Enabled: true",
                  f"        OptimizedEntries: {{Translation: {t}, Rotation: {ro}, Scale: {s}, Shear: {sh}}}",
                  f"        AbsTol: {tol}"]
    p = tmp_path / name
    p.write_text("\n".join(lines) + "\n")
    return p
