"""GPU parity at the benchmarked sizes, against the FP64 oracle.

The other parity tests run small grids so that the oracle's fields can be
compared voxel by voxel. This file checks the LC2 values of the benchmarked
workloads themselves, at their full size and launch shape, so that what only
shows at scale is covered: sampling bands far from the origin, the automatic
z split of a 256^3 grid, 64-bit sums over 16.8 M voxels, and a launch of 512
transforms.

  * 3D 256^3 -> 256^3 at 1 mm, 9^3 patches, 10 % constant ultrasound blocks,
    512 candidate affines in one launch, f16 and bf16 storage (the
    benchmark's main line), with HighResolutionModality Moving and Fixed;
  * 2D 256^2, 7x7 patches, 512 affines per launch, f32;
  * 3D 128^3 -> 96^3, 7^3 patches, 256 affines per launch, f32;
  * 3D 200^3, 7^3 patches, 64 affines per launch, f32 (24-row tiles and one
    row of 16-row tiles for the 8 rows they leave over).

The oracle is fed the same storage-rounded volumes. Tolerance: 1e-5
relative on LC2.
"""
import numpy as np
import pytest

from lc2registration_gb300 import capi, synth
from tests.helpers import oracle_eval, perturbed

pytestmark = pytest.mark.gpu

REL_LC2 = 1e-5


@pytest.fixture(scope="module")
def main_case():
    case = synth.case_3d(seed=2024, mr_size=256, us_size=256, r=4, constant_block_frac=0.1)
    mats = perturbed(case, np.random.default_rng(77), 512, scale=1.0)
    return case, mats


def _check(case, mats, storage, picks, hr_moving=True):
    ctx = capi.Context(case.mode, case.fixed_geom, case.moving_geom, case.virt_spacing, case.r,
                       hr_moving, storage)
    ctx.set_images(case.fixed, case.moving)
    vals = ctx.evaluate_batch(mats)
    one = ctx.evaluate(mats[picks[0]])  # one transform: another launch shape and z split
    ctx.close()
    assert one == vals[picks[0]]
    worst = 0.0
    for i in picks:
        ref = oracle_eval(case, mats[i], storage=storage)
        assert ref > 0.01, (i, ref)
        rel = abs(vals[i] / ref - 1.0)
        worst = max(worst, rel)
        assert rel < REL_LC2, (i, vals[i], ref, rel)
    return worst


@pytest.mark.parametrize("storage", ["f16", "bf16"])
def test_256cubed_batch_of_512_matches_oracle(main_case, storage):
    case, mats = main_case
    _check(case, mats, storage, [0, 1, 2, 255, 510, 511])


def test_256cubed_fixed_modality_matches_oracle(main_case):
    case, mats = main_case
    inv = np.linalg.inv(mats[:128].astype(np.float64)).astype(np.float32)
    swapped = synth.Case(case.mode, case.moving_geom, case.moving, case.fixed_geom, case.fixed,
                         [1.0, 1.0, 1.0], case.r, hr_moving=False, true_params={},
                         true_mat=inv[0])
    _check(swapped, inv, "f16", [0, 63, 127], hr_moving=False)


def test_2d_256sq_batch_matches_oracle():
    case = synth.case_2d(seed=7, size=256, r=3)
    mats = perturbed(case, np.random.default_rng(3), 512)
    _check(case, mats, "f32", list(range(0, 512, 37)) + [511])


def test_3d_128_to_96_batch_matches_oracle():
    case = synth.case_3d(seed=8, mr_size=128, us_size=96, r=3)
    mats = perturbed(case, np.random.default_rng(3), 256)
    _check(case, mats, "f32", [0, 1, 100, 200, 255])


def test_200cubed_split_tiles_match_oracle():
    """A 200-row grid: 24-row tiles over rows 0-191 and one row of 16-row
    tiles over rows 192-199 (8 of its 16 rows outside the grid), radius 3,
    FP32, 64 transforms per launch."""
    case = synth.case_3d(seed=9, mr_size=200, us_size=200, r=3)
    mats = perturbed(case, np.random.default_rng(4), 64)
    _check(case, mats, "f32", [0, 31, 63])
