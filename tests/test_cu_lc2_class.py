"""The reference's LC2 similarity objects, LC2_3D_class and LC2_2D_class
(include/lc2_cu_lc2.hpp): a C++ caller written against the reference's
headers (tests/cpp/lc2_class_eval.cpp) compiles against this header, and on
the GPU its values equal the C ABI's bit for bit -- a context over the same
grid evaluated at the identity -- and the FP64 oracle's within 1e-5."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from lc2registration_gb300 import build as lbuild
from lc2registration_gb300.geometry import Geometry

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = "/usr/local/cuda"


def build_driver(tmpdir) -> str:
    if shutil.which("g++") is None or not os.path.isdir(os.path.join(CUDA, "include")):
        pytest.skip("g++ or CUDA headers missing")
    lib = lbuild.build()
    exe = os.path.join(str(tmpdir), "lc2_class_eval")
    subprocess.run(["g++", "-std=c++14", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(CUDA, "include"),
                    os.path.join(ROOT, "tests", "cpp", "lc2_class_eval.cpp"),
                    "-L", os.path.dirname(lib), "-llc2", "-L", os.path.join(CUDA, "lib64"),
                    "-lcudart", f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", exe], check=True)
    return exe


def test_class_header_compiles(tmp_path):
    build_driver(tmp_path)


def _grid_pair(mode):
    """An ultrasound image and the high-resolution image resampled onto its
    grid at the generating transform (what the reference's interpolators write
    into the object's buffers)."""
    from lc2registration_gb300 import synth
    from tests.helpers import make_context

    if mode == "3D":
        case = synth.case_3d(seed=71, mr_size=40, us_size=32, r=2, blobs=5)
    else:
        case = synth.case_2d(seed=72, size=64, r=3)
    ctx = make_context(case)
    _, f = ctx.evaluate_fields(case.true_mat)
    ctx.close()
    return case, np.ascontiguousarray(case.fixed, np.float32), np.ascontiguousarray(f["M"],
                                                                                     np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["3D", "2D"])
def test_class_matches_c_abi_and_oracle(tmp_path, mode):
    from lc2registration_gb300 import capi
    from oracle import oracle as O

    exe = build_driver(tmp_path)
    case, us, hr = _grid_pair(mode)
    dims = list(case.fixed_geom.dim)
    us.tofile(tmp_path / "us.raw")
    hr.tofile(tmp_path / "hr.raw")
    out = subprocess.run([exe, mode, *map(str, dims), str(case.r), str(tmp_path / "us.raw"),
                          str(tmp_path / "hr.raw"), str(tmp_path)],
                         capture_output=True, text=True, check=True).stdout
    vals = [float(v) for v in out.split()]

    nd = 3 if mode == "3D" else 2
    grid = Geometry(tuple(dims), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0))
    ident = np.eye(nd + 1, dtype=np.float32)
    ctx = capi.Context(mode, grid, grid, [1.0] * nd, case.r)
    ctx.set_images(us, hr)
    ref, f = ctx.evaluate_fields(ident)
    assert vals[0] == ref, (vals[0], ref)  # the object built from host vectors
    n = int(np.prod(dims))
    grad = np.fromfile(tmp_path / "grad.raw", dtype=np.float32, count=n)
    assert np.array_equal(grad, f["G"].ravel())
    if mode == "3D":
        assert vals[1] == 0.0  # zeroed buffers: no valid patch
        wmap = np.fromfile(tmp_path / "wmap.raw", dtype=np.float32, count=n)
        assert np.array_equal(wmap, ctx.weighting_map(ident)[1].ravel())
        mi_ctx = capi.Context(mode, grid, grid, [1.0] * nd, 0)
        mi_ctx.set_images(us, hr)
        assert vals[2] == mi_ctx.evaluate(ident)
        mi_ctx.close()
    else:
        assert vals[1] == ref  # filled through the device pointers
    ctx.close()
    og = O.Geom(list(dims), [1.0, 1.0, 1.0], [0.0, 0.0, 0.0])
    orc = O.lc2_eval(mode, og, us, og, hr, [1.0] * nd, case.r, ident)
    assert abs(vals[0] / orc - 1.0) < 1e-5, (vals[0], orc)
