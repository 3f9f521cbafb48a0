"""GPU parity of the fused kernel of a resampled ultrasound
(HighResolutionModality: Fixed: the MR/CT is the static high-resolution
image, the ultrasound is warped per transform) against the FP64 oracle and
against the generic path (LC2_OPTION_GENERIC), through the C ABI.

Tolerances: LC2 within 1e-5 relative of the oracle;
fused against generic within 1e-6 relative (the two place their sampling
bases differently, so an interpolated value can differ in its last bit and a
quantised ultrasound value by one step); tile heights, batch vs plain: bit-
identical (exact integer sums).
"""
import numpy as np
import pytest

from lc2registration_gb300 import capi
from tests.helpers import make_context, oracle_eval, perturbed
from tests.test_gpu_parity import REL_LC2, _case, _hr_fixed

pytestmark = pytest.mark.gpu

KINDS = ["2d", "2d_r1", "2d_r9", "3d", "3d_r3", "3d_r4", "3d_r5", "3d_r6"]


def _fixed(kind, n, seed=5, scale=0.5):
    """The case with the roles of HighResolutionModality: Fixed and n
    transforms around its true one (inverses of the moving-mode ones)."""
    base = _case(kind)
    mats = perturbed(base, np.random.default_rng(seed), n, scale=scale)
    inv = np.linalg.inv(mats.astype(np.float64)).astype(np.float32)
    case = _hr_fixed(base)
    return case, np.concatenate([case.true_mat[None], inv])


@pytest.mark.parametrize("kind", KINDS)
def test_fixed_fused_matches_oracle(kind):
    case, mats = _fixed(kind, 2)
    ctx = make_context(case)
    got = ctx.evaluate_batch(mats)
    for k in range(len(mats)):
        ref = oracle_eval(case, mats[k], use_boxsum=False)
        assert ref > 0.01
        assert abs(got[k] / ref - 1.0) < REL_LC2, (k, got[k], ref)


@pytest.mark.parametrize("kind", ["2d", "2d_r9", "3d", "3d_r4", "3d_r6"])
def test_fixed_fused_matches_generic_path(kind):
    case, mats = _fixed(kind, 5)
    ctx = make_context(case)
    fused = ctx.evaluate_batch(mats)
    ctx.set_option(capi.OPTION_GENERIC, 1)
    generic = ctx.evaluate_batch(mats)
    ctx.set_option(capi.OPTION_GENERIC, 0)
    np.testing.assert_allclose(fused, generic, rtol=1e-6, atol=0)
    # the generic LC2 of evaluate_fields agrees too
    lc2_fields, _ = ctx.evaluate_fields(mats[0])
    assert abs(lc2_fields / fused[0] - 1.0) < 1e-6


@pytest.mark.parametrize("kind", ["3d", "3d_r4"])
def test_fixed_tile_heights_and_zchunks_bitwise(kind):
    case, mats = _fixed(kind, 3)
    ctx = make_context(case)
    base = ctx.evaluate_batch(mats)
    for rows, zc in [(8, 0), (16, 7), (8, 13)]:
        ctx.set_option(capi.OPTION_TILE_ROWS, rows)
        ctx.set_option(capi.OPTION_ZCHUNK, zc)
        assert np.array_equal(ctx.evaluate_batch(mats), base), (rows, zc)
    ctx.set_option(capi.OPTION_TILE_ROWS, 0)
    ctx.set_option(capi.OPTION_ZCHUNK, 0)


@pytest.mark.parametrize("kind", ["2d", "3d"])
def test_fixed_batch_equals_plain_bitwise(kind):
    case, mats = _fixed(kind, 6)
    ctx = make_context(case, max_batch=3)
    batch = ctx.evaluate_batch(mats)
    plain = np.array([ctx.evaluate(m) for m in mats])
    assert np.array_equal(batch, plain)


@pytest.mark.parametrize("storage", ["f16", "bf16"])
@pytest.mark.parametrize("kind", ["2d", "3d_r4"])
def test_fixed_reduced_storage_matches_oracle_on_rounded_inputs(kind, storage):
    case, mats = _fixed(kind, 2)
    ctx = make_context(case, storage=storage)
    got = ctx.evaluate_batch(mats)
    for k in range(len(mats)):
        ref = oracle_eval(case, mats[k], storage=storage)
        assert abs(got[k] / ref - 1.0) < REL_LC2, (k, got[k], ref)


def test_fixed_autotune_keeps_values():
    """The autotuner picks a tile height among 8, 16 and 24 rows (the
    768-thread kernel on the presampled ultrasound) and the values stay the
    same bits."""
    case, mats = _fixed("3d_r3", 4)
    ctx = make_context(case)
    before = ctx.evaluate_batch(mats)
    rows, zc = ctx.autotune(mats)
    assert rows in (8, 16, 24)
    assert np.array_equal(ctx.evaluate_batch(mats), before)


def test_fixed_degenerate_inputs():
    """Out-of-view transform: the warped ultrasound is 0 everywhere, every
    patch is invalid, LC2 = 0/0 -> 0 on the GPU as in the oracle."""
    case, mats = _fixed("3d", 1)
    away = mats[0].copy()
    away[0, -1] += 1e4
    ctx = make_context(case)
    assert ctx.evaluate(away) == 0.0
    assert oracle_eval(case, away) == 0.0


def test_fixed_2d_wide_perturbations_match_oracle():
    """Transforms spread as far as the benchmark's (scale 1.0), where more of
    the warped ultrasound falls outside its image: fused and generic paths
    both within 1e-5 of the oracle."""
    case, mats = _fixed("2d", 10, seed=11, scale=1.0)
    ctx = make_context(case)
    fused = ctx.evaluate_batch(mats)
    ctx.set_option(capi.OPTION_GENERIC, 1)
    generic = ctx.evaluate_batch(mats)
    for k in range(len(mats)):
        ref = oracle_eval(case, mats[k], use_boxsum=False)
        if ref == 0.0:
            assert fused[k] == 0.0 and generic[k] == 0.0
            continue
        assert abs(fused[k] / ref - 1.0) < REL_LC2, (k, fused[k], ref)
        assert abs(generic[k] / ref - 1.0) < REL_LC2, (k, generic[k], ref)


def test_fixed_replays_graphs_generic_does_not():
    case, mats = _fixed("3d", 3)
    ctx = make_context(case)
    first = ctx.evaluate_batch(mats)  # captured
    g0 = ctx.graph_launches()
    assert np.array_equal(ctx.evaluate_batch(mats), first)
    assert ctx.graph_launches() == g0 + 1
    ctx.set_option(capi.OPTION_GENERIC, 1)
    g1 = ctx.graph_launches()
    ctx.evaluate_batch(mats)
    assert ctx.graph_launches() == g1


def test_fixed_odd_sizes_and_tiny_grids():
    from lc2registration_gb300 import synth
    from lc2registration_gb300.geometry import Geometry

    rng = np.random.default_rng(19)
    for (nx, ny, nz, r) in [(7, 5, 3, 1), (33, 9, 11, 2), (65, 17, 1, 4), (41, 23, 19, 5)]:
        mode = "3D" if nz > 1 else "2D"
        g = Geometry((nx, ny, nz), (1, 1, 1), (0, 0, 0))
        mov = (rng.random((nz, ny, nx)) + 0.2).astype(np.float32)
        fix = rng.random((nz, ny, nx)).astype(np.float32)
        vs = [1.0, 1.0, 1.0][: (3 if mode == "3D" else 2)]
        case = synth.Case(mode, g, fix, g, mov, vs, r, False, {}, None)
        mat = np.eye(4 if mode == "3D" else 3, dtype=np.float32)
        mat[0, -1] = 0.37
        ctx = make_context(case)
        got = ctx.evaluate(mat)
        ref = oracle_eval(case, mat, use_boxsum=False)
        if ref == 0.0:
            assert got == 0.0
        else:
            assert abs(got / ref - 1.0) < REL_LC2, (nx, ny, nz, r, got, ref)


@pytest.mark.parametrize("hr_moving", [True, False])
def test_anisotropic_spacings_match_oracle(hr_moving):
    """Fixed, moving and virtual spacings all different and anisotropic, so
    the virtual grid is neither image's grid."""
    from lc2registration_gb300 import synth
    from lc2registration_gb300.geometry import Geometry, affine3d

    rng = np.random.default_rng(23)
    fg = Geometry((30, 26, 22), (1.1, 0.9, 1.3), (2.0, -1.0, 0.5))
    mg = Geometry((36, 34, 30), (0.95, 1.05, 0.85), (0.0, 0.0, 0.0))
    mr = synth.mr_phantom((30, 34, 36), 6, 1.2, seed=41)
    us = (rng.random((22, 26, 30)) * 0.2 + 0.3).astype(np.float32)
    if hr_moving:
        case = synth.Case("3D", fg, us, mg, mr, [1.2, 0.8, 1.0], 2, True, {}, None)
    else:
        case = synth.Case("3D", mg, mr, fg, us, [1.2, 0.8, 1.0], 2, False, {}, None)
    mats = [affine3d((2.0, -1.5, 1.0), (0.7, -0.4, 0.3), (1.02, 0.98, 1.0), (0.01, 0.0, -0.01),
                     (15.0, 14.0, 13.0), (0, 0, 0)).astype(np.float32)]
    ctx = make_context(case)
    for m in mats:
        got = ctx.evaluate(m)
        ref = oracle_eval(case, m, use_boxsum=False)
        assert ref > 0.0
        assert abs(got / ref - 1.0) < REL_LC2, (got, ref)


def test_fixed_2dto3d_matches_oracle_and_generic():
    """2D-to-3D with HighResolutionModality: Fixed: the frame is the static
    high-resolution image and the volume is sampled trilinearly per
    transform (k_fused_fixed2 with 3D sampling)."""
    base = _case("2dto3d")
    from lc2registration_gb300 import synth

    case = synth.Case(base.mode, base.fixed_geom, base.fixed, base.moving_geom, base.moving,
                      base.virt_spacing, base.r, hr_moving=False, true_params={},
                      true_mat=base.true_mat)
    mats = np.concatenate([case.true_mat[None],
                           perturbed(base, np.random.default_rng(8), 3, scale=0.5)])
    ctx = make_context(case)
    fused = ctx.evaluate_batch(mats)
    ctx.set_option(capi.OPTION_GENERIC, 1)
    generic = ctx.evaluate_batch(mats)
    for k in range(len(mats)):
        ref = oracle_eval(case, mats[k], use_boxsum=False)
        assert ref > 0.0
        assert abs(fused[k] / ref - 1.0) < REL_LC2, (k, fused[k], ref)
        assert abs(generic[k] / ref - 1.0) < REL_LC2, (k, generic[k], ref)
