"""Regenerates the golden fixtures in tests/golden/ from the reference itself.

Runs in the development container only (it needs the reference sources):
`make -C oracle ref` builds, from the reference's own sources,
  * oracle/_ref/mappers_golden -- the reference's transform builders
    (src/Interpolator/spatialMappers.cuh), and
  * oracle/_ref/libref_kernels.so -- the reference's resampling, Sobel,
    weighting-factor and CG-similarity kernels run on the CPU under
    oracle/ref_golden/kernel_emu.cpp;
this script runs them on seeded synthetic inputs and writes
  ref_mappers.txt   transform matrices and inverses,
  ref_lc2_cases.npz inputs, geometry and the reference's per-voxel outputs
                    (U, M, G, weighting factor W, weighted similarity S).

    python tests/golden/make_golden.py
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lc2registration_gb300 import synth  # noqa: E402
from lc2registration_gb300.geometry import Geometry  # noqa: E402
from oracle import oracle as O, refkernels as R  # noqa: E402
from tests.helpers import ogeom  # noqa: E402


def cases():
    """(name, Case) pairs: every mode, both modalities, 3D r=4 takes the
    reference's global-memory similarity kernel."""
    out = [("2d_r3", synth.case_2d(seed=101, size=40, r=3)),
           ("2d_r1", synth.case_2d(seed=102, size=32, r=1)),
           ("3d_r2", synth.case_3d(seed=103, mr_size=26, us_size=20, r=2, blobs=5)),
           ("3d_r3", synth.case_3d(seed=104, mr_size=28, us_size=22, r=3, blobs=5)),
           ("3d_r4", synth.case_3d(seed=105, mr_size=30, us_size=24, r=4, blobs=5))]
    mr = synth.mr_phantom((24, 24, 24), 5, 1.5, seed=106)
    mg = Geometry((24, 24, 24), (1, 1, 1), (0, 0, 0))
    out.append(("2dto3d_r3", synth.frame_stack(mr, mg, 1, seed=107, sides=(36,), spacing=0.5, r=3)[0]))
    c = synth.case_2d(seed=108, size=36, r=2)
    inv = np.linalg.inv(c.true_mat.astype(np.float64)).astype(np.float32)
    out.append(("2d_hrfixed_r2", synth.Case("2D", c.moving_geom, c.moving, c.fixed_geom, c.fixed,
                                            [1.0, 1.0], 2, False, {}, inv)))
    return out


def main():
    ref = os.environ.get("REF", "/root/reference")
    if not os.path.isdir(ref):
        sys.exit(f"reference sources not found at {ref}")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={ref}"],
                   check=True)
    out = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "mappers_golden")], check=True,
                         capture_output=True, text=True).stdout
    with open(os.path.join(HERE, "ref_mappers.txt"), "w") as f:
        f.write(out)
    arrays = {}
    for name, c in cases():
        nd = 2 if c.mode == "2D" else 3
        vg = O.virtual_geom(nd, ogeom(c.fixed_geom), c.virt_spacing)
        res = R.evaluate(c.mode, ogeom(c.fixed_geom), c.fixed, ogeom(c.moving_geom), c.moving, vg,
                         c.true_mat, c.r, c.hr_moving)
        meta = np.array([nd, c.r, int(c.hr_moving), {"2D": 0, "3D": 1, "2DTo3D": 2}[c.mode]],
                        dtype=np.int32)
        geo = np.array([list(c.fixed_geom.dim) + list(c.fixed_geom.spacing) + list(c.fixed_geom.origin),
                        list(c.moving_geom.dim) + list(c.moving_geom.spacing) + list(c.moving_geom.origin),
                        list(vg.dim) + list(vg.spacing) + list(vg.origin)], dtype=np.float64)
        arrays[f"{name}/meta"] = meta
        arrays[f"{name}/geom"] = geo
        arrays[f"{name}/vspacing"] = np.array(list(c.virt_spacing) + [1.0] * (3 - len(c.virt_spacing)))
        arrays[f"{name}/fixed"] = c.fixed
        arrays[f"{name}/moving"] = c.moving
        arrays[f"{name}/mat"] = c.true_mat
        for k in "UMGWS":
            arrays[f"{name}/{k}"] = res[k]
        print(name, c.mode, "virtual", vg.dim, "valid", int((res["W"] > 0).sum()))
    np.savez_compressed(os.path.join(HERE, "ref_lc2_cases.npz"), **arrays)
    print("wrote ref_mappers.txt, ref_lc2_cases.npz")


if __name__ == "__main__":
    main()
