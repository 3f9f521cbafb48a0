"""The reference's registration flow from a parameter file
(Interpolator(yaml) -> Optimizers(yaml) -> Optimize -> ExportResults) through
the C++ drop-in headers, against lc2_register called directly with the same
settings, and the files it writes (RegistrationInfo.log, <name>_result.yaml)."""
import re
import subprocess

import numpy as np
import pytest

from lc2registration_gb300 import capi, synth
from tests.helpers import make_context, write_param_file
from tests.test_yaml import build_register

pytestmark = pytest.mark.gpu

ROUNDS = [("true", "true", "false", "false", "1.0e-4"),
          ("true", "true", "true", "true", "1.0e-4")]


def _flow(text, key):
    m = re.search(rf"^\s*{key}: \{{(.*)\}}$", text, re.M)
    return {k.strip(): float(v) for k, v in (kv.split(":") for kv in m.group(1).split(","))}


def _run(tmp_path, mode, case, lo, hi):
    exe = build_register(tmp_path)
    p = write_param_file(tmp_path, case, rounds=ROUNDS)
    out = subprocess.run([exe, mode, str(p)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    line1, line2 = out.stdout.strip().splitlines()
    params = np.array([float(v) for v in line1.split()])
    sim, evals, result = line2.split()
    init = np.array([0, 0, 0, 1, 1, 0.0]) if mode == "2D" else \
        np.array([0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0.0])
    rounds = [(["translation", "rotation"], 1e-4),
              (["translation", "rotation", "scale", "shear"], 1e-4)]
    ref = capi.register(make_context(case), init, lo, hi, center=case.fixed_geom.center(),
                        direct_entries=["translation"], direct_maxeval=50, rounds=rounds)
    return params, float(sim), int(evals), result, ref


def _check_files(tmp_path, result, params, sim, evals, keys, mode, case):
    text = open(result).read()
    iv = _flow(text, "InitialValues")
    got = np.array([iv[k] for k in keys])
    np.testing.assert_allclose(got, params.astype(np.float32), rtol=1e-6, atol=1e-7)
    assert re.search(r"^\s*IsRegistered: true$", text, re.M)
    assert int(re.search(r"NumEvaluations: (\d+)", text).group(1)) == evals
    assert abs(float(re.search(r"LastSimilarity: (\S+)", text).group(1)) - sim) < 1e-7
    d = 3 if mode == "2D" else 4
    rows = re.findall(r"^\s*-\n((?:\s*- \S+\n){%d})" % d, text, re.M)
    tm = np.array([[float(v) for v in re.findall(r"- (\S+)", r)] for r in rows[-d:]])
    m = capi.params_to_matrix(mode, params, case.fixed_geom.center(), (0, 0, 0))
    np.testing.assert_allclose(tm @ m, np.eye(d), atol=2e-5)
    log = open(tmp_path / "RegistrationInfo.log").read().strip().splitlines()
    assert log[0].startswith("Step,Transform[16]")
    assert len(log) == 1 + 1 + evals        # header, initial row, one row per evaluation
    assert "Enabled: false" in text          # DIRECT and round 0 disabled for a re-run
    if mode == "3D":
        # WriteOut(OptimalMatrix): moving volume with transformed axes/origin, and the matrix
        from tests.test_io import read_nrrd
        fields, body = read_nrrd(tmp_path / "moving_Registered.nrrd")
        np.testing.assert_array_equal(body, case.moving.astype(np.float32).ravel())
        sp, org = np.array(case.moving_geom.spacing), np.array(case.moving_geom.origin)
        dirs = [np.array(v.split(","), float) for v in
                fields["space directions"].strip("()").split(") (")]
        for a in range(3):
            np.testing.assert_allclose(dirs[a], tm[:3, a] * sp[a], rtol=2e-5, atol=2e-5)
        o = np.array(fields["space origin"].strip("()").split(","), float)
        np.testing.assert_allclose(o, tm[:3, :3] @ org + tm[:3, 3], rtol=2e-5, atol=2e-4)
        mat = np.array([[float(v) for v in ln.rstrip(",").split(",")]
                        for ln in open(tmp_path / "MovingToFixed.mat").read().splitlines()])
        np.testing.assert_allclose(mat, tm, rtol=2e-5, atol=2e-5)
    else:
        from tests.test_io import read_png_gray8
        px = read_png_gray8(tmp_path / "moving_Registered.png")
        assert px.shape == (case.fixed_geom.dim[1], case.fixed_geom.dim[0])


def test_register_yaml_2d(tmp_path):
    case = synth.case_2d(seed=1, size=128, r=3)
    lo = np.array([-10, -10, -8, 0.9, 0.9, -0.06])
    hi = np.array([10, 10, 8, 1.1, 1.1, 0.06])
    params, sim, evals, result, ref = _run(tmp_path, "2D", case, lo, hi)
    np.testing.assert_allclose(params, ref["params"], rtol=1e-7, atol=1e-7)
    assert abs(sim / ref["lc2"] - 1) < 1e-7 and evals == ref["evaluations"]
    p = case.true_params
    assert np.abs(params[:2] - np.array(p["trans"])).max() < 0.5
    _check_files(tmp_path, result, params, sim, evals,
                 ["TX", "TY", "R", "ScaleX", "ScaleY", "Shear"], "2D", case)


def test_register_yaml_3d(tmp_path):
    case = synth.case_3d(seed=5, mr_size=40, us_size=32, r=2, blobs=6)
    lo = np.array([-10, -10, -10, -8, -8, -8, 0.9, 0.9, 0.9, -0.05, -0.05, -0.05])
    hi = -lo.copy()
    hi[6:9] = 1.1
    params, sim, evals, result, ref = _run(tmp_path, "3D", case, lo, hi)
    np.testing.assert_allclose(params, ref["params"], rtol=1e-7, atol=1e-7)
    assert abs(sim / ref["lc2"] - 1) < 1e-7 and evals == ref["evaluations"]
    p = case.true_params
    assert np.abs(params[:3] - np.array(p["trans"])).max() < 1.5
    _check_files(tmp_path, result, params, sim, evals,
                 ["TX", "TY", "TZ", "RX", "RY", "RZ", "ScaleX", "ScaleY", "ScaleZ", "ShearX",
                  "ShearY", "ShearZ"], "3D", case)


def test_register_yaml_3d_fixed_modality(tmp_path):
    """HighResolutionModality: Fixed -- the mode of the reference's own 3D
    config: the MR is the fixed (static, high-resolution) volume and the
    ultrasound is warped. The parameter-file flow equals lc2_register called
    directly, on the fused kernel of that modality."""
    base = synth.case_3d(seed=5, mr_size=40, us_size=32, r=2, blobs=6)
    case = synth.Case(base.mode, base.moving_geom, base.moving, base.fixed_geom, base.fixed,
                      list(base.moving_geom.spacing), base.r, hr_moving=False, true_params={},
                      true_mat=np.linalg.inv(base.true_mat.astype(np.float64)).astype(np.float32))
    lo = np.array([-10, -10, -10, -8, -8, -8, 0.9, 0.9, 0.9, -0.05, -0.05, -0.05])
    hi = -lo.copy()
    hi[6:9] = 1.1
    assert "HighResolutionModality: Fixed" in open(
        write_param_file(tmp_path, case, rounds=ROUNDS)).read()
    params, sim, evals, result, ref = _run(tmp_path, "3D", case, lo, hi)
    np.testing.assert_allclose(params, ref["params"], rtol=1e-7, atol=1e-7)
    assert abs(sim / ref["lc2"] - 1) < 1e-7 and evals == ref["evaluations"]
    assert sim > 0.0
    _check_files(tmp_path, result, params, sim, evals,
                 ["TX", "TY", "TZ", "RX", "RY", "RZ", "ScaleX", "ScaleY", "ScaleZ", "ShearX",
                  "ShearY", "ShearZ"], "3D", case)
