"""The YAML subset reader/writer (include/lc2_yaml.hpp) on the reference's
parameter-file schema: parse, re-emit, re-parse."""
import os
import shutil
import subprocess

import pytest

from lc2registration_gb300 import build as lbuild
from lc2registration_gb300 import synth
from tests.helpers import write_param_file

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = "/usr/local/cuda/include"
REF_CONFIGS = "/root/reference/config"


def build_register(tmp_path) -> str:
    if shutil.which("g++") is None or not os.path.isdir(CUDA_INC):
        pytest.skip("g++ or CUDA headers missing")
    lib = lbuild.build()
    exe = os.path.join(str(tmp_path), "register_yaml")
    subprocess.run(["g++", "-std=c++14", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                    "-I", CUDA_INC, os.path.join(ROOT, "tests", "cpp", "register_yaml.cpp"),
                    "-L", os.path.dirname(lib), "-llc2", f"-Wl,-rpath,{os.path.dirname(lib)}",
                    "-o", exe], check=True)
    return exe


def _roundtrip(exe, path, tmp_path):
    once = subprocess.run([exe, str(path)], capture_output=True, text=True, check=True).stdout
    again_path = tmp_path / "again.yaml"
    again_path.write_text(once)
    twice = subprocess.run([exe, str(again_path)], capture_output=True, text=True,
                           check=True).stdout
    assert once == twice
    return once


def test_own_schema_file_roundtrips(tmp_path):
    exe = build_register(tmp_path)
    case = synth.case_3d(seed=3, mr_size=24, us_size=20, r=2, blobs=3)
    p = write_param_file(tmp_path, case)
    out = _roundtrip(exe, p, tmp_path)
    assert "PatchSize: 2" in out and "MaxEvaluations: 50" in out
    assert "OptimizedEntries: {Translation: true, Rotation: true, Scale: true, Shear: true}" in out
    assert "# raw float32" not in out  # comments dropped


@pytest.mark.skipif(not os.path.isdir(REF_CONFIGS), reason="reference configs not present")
@pytest.mark.parametrize("name", ["parameters2d_affine.yaml", "parameters3d_affine.yaml",
                                  "parameters2dTo3d.yaml", "parameters2dTo3d_result.yaml"])
def test_reference_parameter_files_roundtrip(tmp_path, name):
    exe = build_register(tmp_path)
    out = _roundtrip(exe, os.path.join(REF_CONFIGS, name), tmp_path)
    assert "OptimizerSettings:" in out and "TransformMatrix:" in out
    assert "LastSimilarity:" in out
