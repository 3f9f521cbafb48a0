"""Host code under AddressSanitizer + UndefinedBehaviorSanitizer (CPU only):
the FP64 oracle, the optimizers (lc2_minimize), the YAML reader/writer on the
reference's parameter-file schema and the file writers, built with
-fsanitize=address,undefined and run by tests/cpp/sanitize_check.cpp."""
import glob
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_CONFIGS = "/root/reference/config"


def test_host_code_is_clean_under_sanitizers(tmp_path):
    if shutil.which("g++") is None or shutil.which("gcc") is None:
        pytest.skip("gcc/g++ missing")
    san = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer",
           "-g", "-O1"]
    obj = str(tmp_path / "oracle.o")
    r = subprocess.run(["gcc", *san, "-std=c11", "-fopenmp", "-c",
                        os.path.join(ROOT, "oracle", "lc2_oracle.c"), "-o", obj],
                       capture_output=True, text=True)
    if r.returncode != 0 and "asan" in (r.stderr or "").lower():
        pytest.skip("sanitizer runtime missing")
    assert r.returncode == 0, r.stderr
    exe = str(tmp_path / "sanitize_check")
    r = subprocess.run(["g++", *san, "-std=c++17", "-fopenmp",
                        "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"),
                        os.path.join(ROOT, "tests", "cpp", "sanitize_check.cpp"),
                        os.path.join(ROOT, "tests", "cpp", "sanitize_stubs.cpp"),
                        os.path.join(ROOT, "lc2registration_gb300", "csrc", "lc2_optim.cpp"),
                        obj, "-lm", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    configs = sorted(glob.glob(os.path.join(REF_CONFIGS, "*.yaml")))
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0",
               UBSAN_OPTIONS="print_stacktrace=1", OMP_NUM_THREADS="2")
    r = subprocess.run([exe, str(tmp_path), *configs], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0, (r.stdout, r.stderr)
    assert "ERROR: AddressSanitizer" not in r.stderr and "runtime error" not in r.stderr, r.stderr
