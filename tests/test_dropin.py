"""The reference-facing C++ classes (include/lc2_dropin.hpp) build against the
C ABI and drive it the way the reference's optimizer objective does."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from lc2registration_gb300 import build as lbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = "/usr/local/cuda/include"


def build_driver(tmpdir) -> str:
    if shutil.which("g++") is None or not os.path.isdir(CUDA_INC):
        pytest.skip("g++ or CUDA headers missing")
    lib = lbuild.build()
    exe = os.path.join(str(tmpdir), "dropin_eval")
    subprocess.run(["g++", "-std=c++14", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                    "-I", CUDA_INC, os.path.join(ROOT, "tests", "cpp", "dropin_eval.cpp"),
                    "-L", os.path.dirname(lib), "-llc2", f"-Wl,-rpath,{os.path.dirname(lib)}",
                    "-o", exe], check=True)
    return exe


def test_dropin_header_compiles_and_reports_unconfigured(tmp_path):
    exe = build_driver(tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    assert "Please configure the Parameter file!" in out


def _spec(tmp_path, case, params, centred):
    f = tmp_path / "fixed.raw"
    m = tmp_path / "moving.raw"
    case.fixed.astype(np.float32).tofile(f)
    case.moving.astype(np.float32).tofile(m)
    g = lambda geo: " ".join(str(v) for v in (*geo.dim, *geo.spacing, *geo.origin))
    vs = list(case.virt_spacing) + [1.0] * (3 - len(case.virt_spacing))
    lines = [case.mode, g(case.fixed_geom), g(case.moving_geom), " ".join(map(str, vs)),
             f"{case.r} {int(case.hr_moving)} {int(centred)}", str(f), str(m)]
    lines += [" ".join(repr(float(v)) for v in p) for p in params]
    spec = tmp_path / "spec.txt"
    spec.write_text("\n".join(lines) + "\n")
    return spec


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["3D", "2D"])
def test_dropin_matches_c_abi(tmp_path, mode):
    from lc2registration_gb300 import capi, synth
    from lc2registration_gb300.geometry import params_to_matrix

    exe = build_driver(tmp_path)
    if mode == "3D":
        case = synth.case_3d(seed=41, mr_size=40, us_size=30, r=2, blobs=5)
        p = case.true_params
        base = list(p["trans"]) + list(p["rot"]) + list(p["scale"]) + list(p["shear"])
    else:
        case = synth.case_2d(seed=42, size=48, r=3)
        p = case.true_params
        base = list(p["trans"]) + [p["rot"]] + list(p["scale"]) + [p["shear"]]
    rng = np.random.default_rng(0)
    params = [base] + [[v + rng.uniform(-0.5, 0.5) * (0.02 if 0.5 < abs(v) < 1.5 else 1.0)
                        for v in base] for _ in range(3)]
    for centred in (False, True):
        spec = _spec(tmp_path, case, params, centred)
        out = subprocess.run([exe, str(spec)], capture_output=True, text=True, check=True).stdout
        got = np.array([float(v) for v in out.split()])
        ctx = capi.Context(case.mode, case.fixed_geom, case.moving_geom, case.virt_spacing, case.r,
                           case.hr_moving)
        ctx.set_images(case.fixed, case.moving)
        center = case.fixed_geom.center()
        if centred:
            from lc2registration_gb300.geometry import virtual_geometry
            nd = 2 if mode == "2D" else 3
            vg = virtual_geometry(nd, case.fixed_geom, case.virt_spacing)
            mc, vc = case.moving_geom.center(), vg.center()
            shift = [np.float32(mc[a]) - np.float32(vc[a]) for a in range(3)]
        else:
            shift = [0.0, 0.0, 0.0]
        if mode == "2D":
            mats = [capi.affine_2d(q[2], q[0:2], q[3:5], q[5], center[:2], shift[:2]) for q in params]
        else:
            mats = [capi.affine_3d(q[3:6], q[0:3], q[6:9], q[9:12], center, shift) for q in params]
        ref = ctx.evaluate_batch(np.stack(mats))
        assert np.array_equal(got, ref), (got, ref)
