"""Outputs that follow a registration: the weighting map (measure / sigma per
voxel) against the FP64 oracle's fields, and the 2D registered-image warp
against a NumPy restatement of backward bilinear mapping."""
import numpy as np
import pytest

from lc2registration_gb300 import capi, synth
from tests.helpers import make_context, oracle_eval

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["2d", "3d"])
def test_weighting_map_matches_oracle(kind):
    case = (synth.case_2d(seed=41, size=64, r=3) if kind == "2d"
            else synth.case_3d(seed=42, mr_size=40, us_size=32, r=2, blobs=6))
    ctx = make_context(case)
    v, wmap = ctx.weighting_map(case.true_mat)
    ref_v, f = oracle_eval(case, case.true_mat, want_fields=True)
    assert abs(v / ref_v - 1) < 1e-5
    s = f["sigma"]
    ref = np.where(s > 1e-6, f["measure"] / np.where(s > 1e-6, s, 1.0), 0.0)
    assert np.all(wmap[s <= 1e-6] == 0.0)
    np.testing.assert_allclose(wmap, ref, atol=2e-4 * max(1.0, np.abs(ref).max()))
    assert np.all((wmap >= 0) & (wmap <= 1.0 + 1e-5))  # measure <= sigma (R^2 <= 1)


def _warp_ref(src, dst_shape, C):
    sh, sw = src.shape
    A = np.array([[C[0], C[1], C[2]], [C[3], C[4], C[5]], [0, 0, 1.0]])
    inv = np.linalg.inv(A)
    yy, xx = np.mgrid[0:dst_shape[0], 0:dst_shape[1]].astype(np.float64)
    sx = inv[0, 0] * xx + inv[0, 1] * yy + inv[0, 2]
    sy = inv[1, 0] * xx + inv[1, 1] * yy + inv[1, 2]
    inside = (sx >= 0) & (sy >= 0) & (sx <= sw - 1) & (sy <= sh - 1)
    x0 = np.clip(np.floor(sx).astype(int), 0, sw - 1)
    y0 = np.clip(np.floor(sy).astype(int), 0, sh - 1)
    x1, y1 = np.minimum(x0 + 1, sw - 1), np.minimum(y0 + 1, sh - 1)
    fx, fy = sx - x0, sy - y0
    top = src[y0, x0] + fx * (src[y0, x1] - src[y0, x0])
    bot = src[y1, x0] + fx * (src[y1, x1] - src[y1, x0])
    out = np.where(inside, top + fy * (bot - top), 0.0)
    edge = ((np.abs(sx) < 1e-3) | (np.abs(sy) < 1e-3) | (np.abs(sx - (sw - 1)) < 1e-3)
            | (np.abs(sy - (sh - 1)) < 1e-3))
    return out, edge


def test_warp_affine_2d_matches_backward_bilinear():
    rng = np.random.default_rng(3)
    src = rng.random((45, 61)).astype(np.float32) * 200
    th = np.deg2rad(7.0)
    C = [1.05 * np.cos(th), -np.sin(th), 6.3, np.sin(th), 0.97 * np.cos(th), -4.1]
    got = capi.warp_affine_2d(src, (50, 70), C)
    ref, edge = _warp_ref(src.astype(np.float64), (50, 70), C)
    np.testing.assert_allclose(got[~edge], ref[~edge], atol=2e-3)
    assert (got == 0).sum() > 0 and (got > 0).sum() > 1000
    ident = capi.warp_affine_2d(src, src.shape, [1, 0, 0, 0, 1, 0])
    np.testing.assert_array_equal(ident, src)
    with pytest.raises(capi.LC2Error, match="SINGULAR"):
        capi.warp_affine_2d(src, (10, 10), [1, 2, 0, 2, 4, 0])
