"""Normalised mutual information (PatchSize 0, 3D): the GPU value equals the
oracle's binning/entropy rule applied to the same warped volume (exact
histogram), matches the FP64 oracle end to end, peaks at the generating
transform, and drives a registration that maximises it."""
import numpy as np
import pytest

from lc2registration_gb300 import capi, synth
from oracle import oracle as O
from tests.helpers import ogeom, perturbed

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    return synth.case_3d(seed=31, mr_size=48, us_size=40, r=2, blobs=6)


def _ctx(case, patch, storage="f32", hr_moving=True):
    c = capi.Context("3D", case.fixed_geom, case.moving_geom, case.virt_spacing, patch,
                     hr_moving, storage)
    c.set_images(case.fixed, case.moving)
    return c


def test_histogram_is_exact_on_the_same_warped_volume(case):
    mi = _ctx(case, 0)
    lc = _ctx(case, 2)  # its field dump gives the same warped volume
    for m in perturbed(case, np.random.default_rng(0), 4):
        v = mi.evaluate(m)
        _, f = lc.evaluate_fields(m)
        ref = O.nmi(f["U"], f["M"])
        assert abs(v - ref) < 1e-12 * ref, (v, ref)


def test_matches_fp64_oracle_and_peaks_at_truth(case):
    mi = _ctx(case, 0)
    mats = np.concatenate([perturbed(case, np.random.default_rng(1), 6), case.true_mat[None]])
    got = mi.evaluate_batch(mats)
    for m, g in zip(mats, got):
        ref = O.nmi_eval(ogeom(case.fixed_geom), case.fixed, ogeom(case.moving_geom),
                         case.moving, case.virt_spacing, m)
        assert abs(g / ref - 1) < 1e-4, (g, ref)
    assert got[-1] == got.max()
    np.testing.assert_array_equal(got, [mi.evaluate(m) for m in mats])  # batch == plain


def test_high_res_fixed_and_storage(case):
    m = case.true_mat
    hf = _ctx(case, 0, hr_moving=False)
    _, f = _ctx(case, 2, hr_moving=False).evaluate_fields(m)
    assert abs(hf.evaluate(m) - O.nmi(f["U"], f["M"])) < 1e-12
    h16 = _ctx(case, 0, "f16")
    assert abs(h16.evaluate(m) / _ctx(case, 0).evaluate(m) - 1) < 1e-2


def test_registration_maximises_nmi(case):
    mi = _ctx(case, 0)
    c = case.fixed_geom.center()
    init = np.array([0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0.0])
    lo = np.array([-10, -10, -10, -8, -8, -8, 0.9, 0.9, 0.9, -0.05, -0.05, -0.05])
    hi = -lo.copy()
    hi[6:9] = 1.1
    res = capi.register(mi, init, lo, hi, center=c, direct_entries=["translation"],
                        direct_maxeval=60, rounds=[(["translation", "rotation"], 1e-3)])
    start = mi.evaluate(capi.params_to_matrix("3D", init, c))
    assert res["lc2"] > start
    assert np.abs(res["params"][:3] - np.array(case.true_params["trans"])).max() < 2.0


def test_mi_rejected_outside_3d():
    case2 = synth.case_2d(seed=32, size=48, r=3)
    with pytest.raises(capi.LC2Error, match="UNSUPPORTED"):
        capi.Context("2D", case2.fixed_geom, case2.moving_geom, case2.virt_spacing, 0)


@pytest.mark.parametrize("hr_moving", [True, False])
def test_shared_table_histogram_is_exact(hr_moving):
    """A 160^3 grid: batches merge each CTA's counts in the histogram
    kernel's shared table (a CTA's voxels are under 0.5 % of the grid), a
    single evaluation adds to the global histogram directly; both give the
    same bits, and the value equals the binning rule applied to the same
    warped volume, in both HighResolutionModality settings (the histogram's
    two key layouts)."""
    big = synth.case_3d(seed=33, mr_size=168, us_size=160, r=2, blobs=8)
    mats = np.concatenate([big.true_mat[None], perturbed(big, np.random.default_rng(7), 7)])
    if not hr_moving:
        big = synth.Case(big.mode, big.moving_geom, big.moving, big.fixed_geom, big.fixed,
                         [1.0, 1.0, 1.0], big.r, hr_moving=False, true_params={},
                         true_mat=np.linalg.inv(big.true_mat.astype(np.float64)).astype(np.float32))
        mats = np.linalg.inv(mats.astype(np.float64)).astype(np.float32)
    mi = _ctx(big, 0, hr_moving=hr_moving)
    batch = mi.evaluate_batch(mats)
    np.testing.assert_array_equal(batch, [mi.evaluate(m) for m in mats])
    lc = _ctx(big, 2, hr_moving=hr_moving)
    for k in (0, 3):
        _, f = lc.evaluate_fields(mats[k])
        ref = O.nmi(f["U"], f["M"])
        assert abs(batch[k] - ref) < 1e-12 * ref, (k, batch[k], ref)
