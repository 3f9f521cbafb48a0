"""Times the reference's own LC2 kernels on the GPU for the benchmark workloads.

Measurement infrastructure, not product code. Writes the seeded synthetic
inputs of the benchmark (the same generator calls and seeds as bench.py) to
raw float32 files, runs oracle/_ref/ref_gpu_time (built on the GPU host by
`make -C oracle refgpu`, which needs the files `make -C oracle ref` placed in
oracle/_ref/) once per workload, and prints one JSON line per workload:
milliseconds per plain evaluation of the reference's launch sequence
(oracle/ref_golden/ref_gpu_time.cu) and its LC2 value.

    python oracle/ref_golden/ref_gpu_time.py [--evals 3] [--out FILE]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lc2registration_gb300 import synth  # noqa: E402
from lc2registration_gb300.geometry import virtual_geometry  # noqa: E402

BIN = os.path.join(ROOT, "oracle", "_ref", "ref_gpu_time")


def workloads():
    """(name, case): the bench's main 256^3 line at FP32 (the reference's only
    storage type) and its two small configurations."""
    return [
        ("2d_256_r3", synth.case_2d(seed=7, size=256, r=3)),
        ("3d_128_96_r3", synth.case_3d(seed=8, mr_size=128, us_size=96, r=3)),
        ("3d_256_r4", synth.case_3d(seed=2024, mr_size=256, us_size=256, r=4,
                                    constant_block_frac=0.1)),
    ]


def _geom_line(g, path=None):
    d = list(g.dim) + [1] * (3 - len(g.dim))
    s = list(g.spacing) + [1.0] * (3 - len(g.spacing))
    o = list(g.origin) + [0.0] * (3 - len(g.origin))
    vals = [str(int(v)) for v in d] + [repr(float(v)) for v in s] + [repr(float(v)) for v in o]
    return " ".join(vals + ([path] if path else []))


def run_case(name, case, evals, tmp, with_ours=True):
    nd = 2 if case.mode == "2D" else 3
    fpath = os.path.join(tmp, f"{name}_fixed.raw")
    mpath = os.path.join(tmp, f"{name}_moving.raw")
    np.ascontiguousarray(case.fixed, dtype=np.float32).tofile(fpath)
    np.ascontiguousarray(case.moving, dtype=np.float32).tofile(mpath)
    vg = virtual_geometry(nd, case.fixed_geom, case.virt_spacing)
    mat = np.asarray(case.true_mat, dtype=np.float32).ravel()
    lines = [str(nd), _geom_line(case.fixed_geom, fpath), _geom_line(case.moving_geom, mpath),
             _geom_line(vg), f"{1 if case.hr_moving else 0} {case.r} {evals}",
             " ".join(repr(float(v)) for v in mat)]
    cpath = os.path.join(tmp, f"{name}.case")
    with open(cpath, "w") as f:
        f.write("\n".join(lines) + "\n")
    out = subprocess.run([BIN, cpath], capture_output=True, text=True, check=True).stdout
    res = json.loads(out.strip().splitlines()[-1])
    res["workload"] = name
    if with_ours:
        # the same evaluation through this library (FP32 storage), for comparison
        from lc2registration_gb300 import capi

        ctx = capi.Context(case.mode, case.fixed_geom, case.moving_geom, case.virt_spacing, case.r,
                           case.hr_moving, "f32")
        ctx.set_images(case.fixed, case.moving)
        res["lc2_this_library"] = float(ctx.evaluate(case.true_mat))
        ctx.close()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--evals", type=int, default=3)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    if not os.path.exists(BIN):
        sys.exit(f"{BIN} missing: run `make -C oracle refgpu` on the GPU host first")
    rows = []
    with tempfile.TemporaryDirectory() as tmp:
        for name, case in workloads():
            res = run_case(name, case, args.evals, tmp)
            rows.append(res)
            print(json.dumps(res), flush=True)
    if args.out:
        with open(args.out, "w") as f:
            json.dump(rows, f, indent=1)


if __name__ == "__main__":
    main()
