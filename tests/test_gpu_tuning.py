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
    for rows in (8, 16):
        ctx.set_option(capi.OPTION_TILE_ROWS, rows)
        for zc in (0, 6, 7, 13, 40, 1000):
            ctx.set_option(capi.OPTION_ZCHUNK, zc)
            np.testing.assert_array_equal(ctx.evaluate_batch(mats), ref)


def test_autotune_keeps_results(case3d):
    ctx = make_context(case3d, "f16")
    mats = perturbed(case3d, np.random.default_rng(2), 16)
    ref = ctx.evaluate_batch(mats)
    rows, zc = ctx.autotune(mats)
    assert rows in (8, 16) and zc >= 0
    np.testing.assert_array_equal(ctx.evaluate_batch(mats), ref)


def test_tile_rows_16_rejected_for_large_3d_radius():
    case = synth.case_3d(seed=22, mr_size=40, us_size=32, r=5, blobs=4)
    ctx = make_context(case)
    with pytest.raises(capi.LC2Error, match="UNSUPPORTED"):
        ctx.set_option(capi.OPTION_TILE_ROWS, 16)
    rows, _ = ctx.autotune(perturbed(case, np.random.default_rng(3), 2))
    assert rows == 8


def test_2d_context_graphs():
    case = synth.case_2d(seed=23, size=80, r=3)
    ctx = make_context(case)
    mats = perturbed(case, np.random.default_rng(4), 7)
    got = ctx.evaluate_batch(mats)
    np.testing.assert_array_equal(got, _staged(ctx, mats))
    np.testing.assert_array_equal([ctx.evaluate(m) for m in mats], got)
    assert ctx.autotune(mats) == (16, 0)


@pytest.mark.parametrize("r", [1, 2, 4])
def test_warp_specialised_kernel_equals_single_role(r):
    case = synth.case_3d(seed=24 + r, mr_size=48, us_size=40, r=r, blobs=6)
    ctx = make_context(case, "f16")
    mats = perturbed(case, np.random.default_rng(5), 9)
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
