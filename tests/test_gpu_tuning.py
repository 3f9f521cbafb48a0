"""Launch options never change a result: CUDA-graph replay of
lc2_evaluate_batch, explicit z-chunk lengths, tile heights and the autotuner's
choice all give the same LC2 values, bit for bit (every sum is exact)."""
import numpy as np
import pytest

from lc2registration_gb300 import capi, synth
from tests.helpers import make_context, perturbed

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case3d():
    return synth.case_3d(seed=21, mr_size=48, us_size=40, r=2, blobs=6)


def _staged(ctx, mats):
    ctx.stage(mats)
    ctx.launch(len(mats))
    return ctx.fetch(len(mats))


def test_graph_replay_equals_staged_path(case3d):
    ctx = make_context(case3d)
    rng = np.random.default_rng(0)
    for count in (1, 5, 5, 12, 1):
        mats = perturbed(case3d, rng, count)
        g0 = ctx.graph_launches()
        got = ctx.evaluate_batch(mats)
        assert ctx.graph_launches() == g0 + 1
        np.testing.assert_array_equal(got, _staged(ctx, mats))
    ctx.set_option(capi.OPTION_GRAPHS, 0)
    mats = perturbed(case3d, rng, 5)
    g0 = ctx.graph_launches()
    np.testing.assert_array_equal(ctx.evaluate_batch(mats), _staged(ctx, mats))
    assert ctx.graph_launches() == g0


def test_zchunk_and_tile_rows_do_not_change_results(case3d):
    ctx = make_context(case3d)
    mats = perturbed(case3d, np.random.default_rng(1), 6)
    ref = ctx.evaluate_batch(mats)
    for rows in (8, 16, 24):
        ctx.set_option(capi.OPTION_TILE_ROWS, rows)
        for zc in (0, 6, 7, 13, 40, 1000):
            ctx.set_option(capi.OPTION_ZCHUNK, zc)
            np.testing.assert_array_equal(ctx.evaluate_batch(mats), ref)


def test_autotune_keeps_results(case3d):
    ctx = make_context(case3d, "f16")
    mats = perturbed(case3d, np.random.default_rng(2), 16)
    ref = ctx.evaluate_batch(mats)
    rows, zc = ctx.autotune(mats)
    assert rows in (8, 16, 24) and zc >= 0
    np.testing.assert_array_equal(ctx.evaluate_batch(mats), ref)


def test_tile_rows_16_rejected_for_large_3d_radius():
    case = synth.case_3d(seed=22, mr_size=40, us_size=32, r=5, blobs=4)
    ctx = make_context(case)
    for rows in (16, 24):
        with pytest.raises(capi.LC2Error, match="UNSUPPORTED"):
            ctx.set_option(capi.OPTION_TILE_ROWS, rows)
    rows, _ = ctx.autotune(perturbed(case, np.random.default_rng(3), 2))
    assert rows == 8


def test_2d_context_graphs():
    case = synth.case_2d(seed=23, size=80, r=3)
    ctx = make_context(case)
    mats = perturbed(case, np.random.default_rng(4), 7)
    got = ctx.evaluate_batch(mats)
    np.testing.assert_array_equal(got, _staged(ctx, mats))
    np.testing.assert_array_equal([ctx.evaluate(m) for m in mats], got)
    assert ctx.autotune(mats) == (0, 0)  # 2D: tile height chosen per launch
    for rows in (16, 32, 0):
        ctx.set_option(capi.OPTION_TILE_ROWS, rows)
        np.testing.assert_array_equal(ctx.evaluate_batch(mats), got)


@pytest.mark.parametrize("r", [1, 2, 4])
def test_warp_specialised_kernel_equals_single_role(r):
    case = synth.case_3d(seed=24 + r, mr_size=48, us_size=40, r=r, blobs=6)
    ctx = make_context(case, "f16")
    mats = perturbed(case, np.random.default_rng(5), 9)
    ctx.set_option(capi.OPTION_PRESAMPLE, 0)  # the single-role kernel resampling in place
    ref = ctx.evaluate_batch(mats)
    ctx.set_option(capi.OPTION_PIPELINE, 1)
    for zc in (0, 9, 40):
        ctx.set_option(capi.OPTION_ZCHUNK, zc)
        np.testing.assert_array_equal(ctx.evaluate_batch(mats), ref)
        np.testing.assert_array_equal(_staged(ctx, mats), ref)


def test_stream_priority_keeps_results(case3d):
    ctx = make_context(case3d)
    mats = perturbed(case3d, np.random.default_rng(6), 4)
    ref = ctx.evaluate_batch(mats)
    ctx.set_option(capi.OPTION_STREAM_PRIORITY, -1000)
    np.testing.assert_array_equal(ctx.evaluate_batch(mats), ref)
    np.testing.assert_array_equal(_staged(ctx, mats), ref)


@pytest.mark.parametrize("r", [1, 2, 3, 4])
def test_tile_heights_agree_across_sampling_bands(r):
    """A virtual grid 110 rows high spans three 48-row sampling bands (the
    rows that fix a tile's sampling base): 8-, 16- and 24-row tiles, whose
    tiles start at different offsets inside a band, give the same bits, and
    the LC2 values match the oracle, at every radius with 24-row tiles."""
    from lc2registration_gb300.geometry import Geometry, affine3d
    from tests.helpers import oracle_eval
    from tests.test_gpu_parity import REL_LC2

    mg = Geometry((64, 128, 24), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0))
    mr = synth.mr_phantom((24, 128, 64), 8, 1.5, seed=33)
    ug = Geometry((40, 110, 12), (1.0, 1.0, 1.0), (12.0, 9.0, 6.0))
    p = dict(rot=[2.0, -3.0, 4.0], trans=[1.5, -2.0, 0.5], scale=[1.02, 0.98, 1.0],
             shear=[0.01, 0.0, -0.01])
    mat = affine3d(p["rot"], p["trans"], p["scale"], p["shear"], ug.center(), (0.0, 0.0, 0.0))
    us = synth.us_from_mr(mr, mg, ug, mat, 33)
    case = synth.Case("3D", ug, us, mg, mr, [1.0, 1.0, 1.0], r, True, p, mat.astype(np.float32))
    mats = np.concatenate([case.true_mat[None], perturbed(case, np.random.default_rng(4), 3)])
    ctx = make_context(case)
    ref = None
    for rows in (24, 16, 8):
        ctx.set_option(capi.OPTION_TILE_ROWS, rows)
        got = ctx.evaluate_batch(mats)
        if ref is None:
            ref = got
        np.testing.assert_array_equal(got, ref)
    for k in range(len(mats)):
        want = oracle_eval(case, mats[k], use_boxsum=False)
        assert want > 0.01
        assert abs(ref[k] / want - 1.0) < REL_LC2, (k, ref[k], want)


@pytest.mark.parametrize("kind,storage", [("2d_r5", "f32"), ("2d_r6", "bf16"),
                                          ("2dto3d_r4", "f16")])
def test_2d_tile_heights_agree_and_match_oracle(kind, storage):
    """2D and 2D-to-3D contexts of radius 4-6 run 32-row tiles on large
    launches and 16-row tiles on small ones; both sample from the same
    32-row band, so the choice never changes a bit, and LC2 matches the
    oracle."""
    from lc2registration_gb300.geometry import Geometry
    from tests.helpers import oracle_eval
    from tests.test_gpu_parity import REL_LC2

    if kind == "2d_r5":
        case = synth.case_2d(seed=14, size=100, r=5)
    elif kind == "2d_r6":
        case = synth.case_2d(seed=15, size=90, r=6)
    else:
        mr = synth.mr_phantom((40, 40, 40), 6, 1.5, seed=34)
        mg = Geometry((40, 40, 40), (1, 1, 1), (0, 0, 0))
        case = synth.frame_stack(mr, mg, 1, seed=35, sides=(70,), spacing=0.5, r=4)[0]
    mats = np.concatenate([case.true_mat[None], perturbed(case, np.random.default_rng(6), 3)])
    ctx = make_context(case, storage)
    ref = ctx.evaluate_batch(mats)
    for rows in (32, 16, 0):
        ctx.set_option(capi.OPTION_TILE_ROWS, rows)
        np.testing.assert_array_equal(ctx.evaluate_batch(mats), ref)
        np.testing.assert_array_equal([ctx.evaluate(m) for m in mats[:2]], ref[:2])
    for k in range(len(mats)):
        want = oracle_eval(case, mats[k], storage=storage, use_boxsum=False)
        assert want > 0.01
        assert abs(ref[k] / want - 1.0) < REL_LC2, (k, ref[k], want)


@pytest.mark.parametrize("r,storage", [(1, "f32"), (3, "f16"), (4, "bf16")])
def test_presample_forms(r, storage):
    """LC2_OPTION_PRESAMPLE: the resample pass (1, the default) gives the
    same bits whatever the tile height, z chunk, group size or batch, agrees
    with the in-kernel resampling (0) to FP32 resampling rounding and with the
    FP64 oracle to 1e-5; other values are refused."""
    from tests.helpers import oracle_eval

    case = synth.case_3d(seed=60 + r, mr_size=48, us_size=40, r=r, blobs=6)
    ctx = make_context(case, storage)
    mats = perturbed(case, np.random.default_rng(r), 11)
    ref = ctx.evaluate_batch(mats)
    np.testing.assert_array_equal([ctx.evaluate(m) for m in mats[:3]], ref[:3])
    with pytest.raises(capi.LC2Error, match="INVALID_ARGUMENT"):
        ctx.set_option(capi.OPTION_PRESAMPLE, 2)
    ctx.set_option(capi.OPTION_PRESAMPLE, 1)
    for rows in (16, 24, 8) if r <= 4 else (8,):
        ctx.set_option(capi.OPTION_TILE_ROWS, rows)
        for zc in (0, 7):
            ctx.set_option(capi.OPTION_ZCHUNK, zc)
            np.testing.assert_array_equal(ctx.evaluate_batch(mats), ref)
    np.testing.assert_array_equal(_staged(ctx, mats), ref)
    ctx.set_option(capi.OPTION_TILE_ROWS, 0)
    ctx.set_option(capi.OPTION_ZCHUNK, 0)
    ctx.set_option(capi.OPTION_PRESAMPLE, 0)
    inkernel = ctx.evaluate_batch(mats)
    assert np.max(np.abs(inkernel / ref - 1.0)) < 2e-6
    for k in (0, 10):
        want = oracle_eval(case, mats[k], storage=storage)
        assert abs(ref[k] / want - 1.0) < 1e-5, (k, ref[k], want)


@pytest.mark.parametrize("r,storage", [(2, "f32"), (4, "f16")])
def test_presample_fixed_modality(r, storage):
    """HighResolutionModality: Fixed with the warped ultrasound presampled (the
    default for 3D): the same bits whatever the tile height (the 768-thread
    kernel at 24 rows), z chunk or batch,
    within FP32 resampling rounding of the in-kernel resampling, and within
    1e-5 of the FP64 oracle."""
    from tests.helpers import oracle_eval

    base = synth.case_3d(seed=70 + r, mr_size=48, us_size=40, r=r, blobs=6)
    inv = np.linalg.inv(base.true_mat.astype(np.float64)).astype(np.float32)
    case = synth.Case(base.mode, base.moving_geom, base.moving, base.fixed_geom, base.fixed,
                      [1.0, 1.0, 1.0], r, hr_moving=False, true_params={}, true_mat=inv)
    ctx = make_context(case, storage)
    mats = np.linalg.inv(perturbed(base, np.random.default_rng(r), 9).astype(np.float64))
    mats = mats.astype(np.float32)
    ref = ctx.evaluate_batch(mats)
    np.testing.assert_array_equal([ctx.evaluate(m) for m in mats[:2]], ref[:2])
    for rows in (16, 24, 8):
        ctx.set_option(capi.OPTION_TILE_ROWS, rows)
        for zc in (0, 7):
            ctx.set_option(capi.OPTION_ZCHUNK, zc)
            np.testing.assert_array_equal(ctx.evaluate_batch(mats), ref)
    ctx.set_option(capi.OPTION_TILE_ROWS, 0)
    ctx.set_option(capi.OPTION_ZCHUNK, 0)
    ctx.set_option(capi.OPTION_PRESAMPLE, 0)
    inkernel = ctx.evaluate_batch(mats)
    assert np.max(np.abs(inkernel / ref - 1.0)) < 2e-6
    for k in (0, 8):
        want = oracle_eval(case, mats[k], storage=storage)
        assert abs(ref[k] / want - 1.0) < 1e-5, (k, ref[k], want)


def test_graph_replay_counts_its_kernels():
    """A graph replay adds to lc2_launch_count the kernels that the same calls
    issue one by one (with the presampled form: resample pass, moments pass
    and the finalizing kernel), not a fixed count per graph."""
    case = synth.case_3d(seed=82, mr_size=48, us_size=40, r=2, blobs=6)
    ctx = make_context(case)
    rng = np.random.default_rng(2)
    mats = perturbed(case, rng, 11)
    ctx.set_option(capi.OPTION_GRAPHS, 0)
    n0 = ctx.launch_count()
    ref = ctx.evaluate_batch(mats)
    direct = ctx.launch_count() - n0
    assert direct >= 3
    ctx.set_option(capi.OPTION_GRAPHS, 1)
    np.testing.assert_array_equal(ctx.evaluate_batch(mats), ref)  # captures, then replays
    n0 = ctx.launch_count()
    g0 = ctx.graph_launches()
    np.testing.assert_array_equal(ctx.evaluate_batch(mats), ref)
    assert ctx.graph_launches() == g0 + 1
    assert ctx.launch_count() - n0 == direct
    ctx.close()


@pytest.mark.parametrize("hr_moving", [True, False])
def test_presample_groups_do_not_change_values(hr_moving):
    """A batch larger than the presample buffer (64 slots at this size) runs
    as several groups, sized to fill whole waves of the device; every
    transform's value equals its value in a batch of one group, bit for bit,
    for both HighResolutionModality settings."""
    base = synth.case_3d(seed=90, mr_size=40, us_size=32, r=2, blobs=5)
    if hr_moving:
        case = base
        mats = perturbed(case, np.random.default_rng(5), 150)
    else:
        inv = np.linalg.inv(base.true_mat.astype(np.float64)).astype(np.float32)
        case = synth.Case(base.mode, base.moving_geom, base.moving, base.fixed_geom, base.fixed,
                          [1.0, 1.0, 1.0], 2, hr_moving=False, true_params={}, true_mat=inv)
        mats = np.linalg.inv(perturbed(base, np.random.default_rng(5), 150).astype(np.float64))
        mats = mats.astype(np.float32)
    ctx = make_context(case)
    whole = ctx.evaluate_batch(mats)
    parts = np.concatenate([ctx.evaluate_batch(mats[i:i + 50]) for i in range(0, 150, 50)])
    np.testing.assert_array_equal(whole, parts)
    np.testing.assert_array_equal([ctx.evaluate(mats[k]) for k in (0, 77, 149)], whole[[0, 77, 149]])
    ctx.close()


@pytest.mark.parametrize("us,r", [(20, 2), (45, 4), (40, 2), (52, 3)])
def test_tall_tiles_on_any_grid_height(us, r):
    """The 24-row moments kernel on grid heights that it covers alone (20,
    45: the last tile partly outside) or together with one row of 16-row
    tiles (40 = 24 + 16, 52 = 48 + 4) gives the bits of the 16-row kernel."""
    case = synth.case_3d(seed=95 + us, mr_size=us + 8, us_size=us, r=r, blobs=5)
    ctx = make_context(case, "f16")
    mats = perturbed(case, np.random.default_rng(us), 7)
    ctx.set_option(capi.OPTION_TILE_ROWS, 16)
    ref = ctx.evaluate_batch(mats)
    ctx.set_option(capi.OPTION_TILE_ROWS, 24)
    np.testing.assert_array_equal(ctx.evaluate_batch(mats), ref)
    np.testing.assert_array_equal([ctx.evaluate(m) for m in mats[:2]], ref[:2])
    ctx.close()


@pytest.mark.parametrize("us,r", [(20, 2), (45, 4), (40, 3)])
def test_tall_tiles_fixed_modality(us, r):
    """The 24-row kernel of HighResolutionModality: Fixed, alone (20, 45 rows)
    or with a row of 16-row tiles (40 = 24 + 16), gives the bits of the 16-row
    kernel."""
    base = synth.case_3d(seed=97 + us, mr_size=us + 8, us_size=us, r=r, blobs=5)
    inv = np.linalg.inv(base.true_mat.astype(np.float64)).astype(np.float32)
    case = synth.Case(base.mode, base.moving_geom, base.moving, base.fixed_geom, base.fixed,
                      [1.0, 1.0, 1.0], r, hr_moving=False, true_params={}, true_mat=inv)
    ctx = make_context(case, "f16")
    mats = np.linalg.inv(perturbed(base, np.random.default_rng(us), 7).astype(np.float64))
    mats = mats.astype(np.float32)
    ctx.set_option(capi.OPTION_TILE_ROWS, 16)
    ref = ctx.evaluate_batch(mats)
    ctx.set_option(capi.OPTION_TILE_ROWS, 24)
    np.testing.assert_array_equal(ctx.evaluate_batch(mats), ref)
    np.testing.assert_array_equal([ctx.evaluate(m) for m in mats[:2]], ref[:2])
    ctx.close()


def test_weighting_map_on_tall_tiles():
    """The per-voxel measure written by the moments pass (lc2_weighting_map)
    is the same with 24-row tiles plus a row of 16-row tiles (a 40-row grid)
    as with 16-row tiles alone."""
    case = synth.case_3d(seed=99, mr_size=48, us_size=40, r=3, blobs=5)
    ctx = make_context(case, "f16")
    ctx.set_option(capi.OPTION_TILE_ROWS, 16)
    v16, m16 = ctx.weighting_map(case.true_mat)
    ctx.set_option(capi.OPTION_TILE_ROWS, 24)
    v24, m24 = ctx.weighting_map(case.true_mat)
    assert v24 == v16
    np.testing.assert_array_equal(m24, m16)
    assert np.count_nonzero(m16) > 0
    ctx.close()
