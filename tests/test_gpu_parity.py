"""GPU parity of the CUDA LC2 path against the FP64 oracle (through the C ABI).

Tolerances:
  * LC2 value: 1e-5 relative to the oracle;
  * warped image M and its Sobel magnitude G: 2e-5 of the image's range
    (FP32 resampling vs FP64; coordinates agree to ~1e-6 voxel);
  * sigma: 1e-5 relative where both are non-zero, identical zero pattern
    except for voxels within 1e-4 of the 1e-6 variance threshold;
  * batched vs plain evaluation: bit-identical (exact integer reductions).
"""
import numpy as np
import pytest

from lc2registration_gb300 import capi, synth
from lc2registration_gb300.geometry import Geometry, affine3d
from tests.helpers import make_context, oracle_eval, perturbed, round_storage

pytestmark = pytest.mark.gpu

REL_LC2 = 1e-5


def _case(kind):
    if kind == "2d":
        return synth.case_2d(seed=11, size=64, r=3)
    if kind == "2d_r1":
        return synth.case_2d(seed=12, size=40, r=1)
    if kind == "2d_r9":
        return synth.case_2d(seed=13, size=72, r=9)
    if kind == "3d":
        return synth.case_3d(seed=21, mr_size=44, us_size=34, r=2, blobs=6, blur=1.5)
    if kind == "3d_r3":
        return synth.case_3d(seed=22, mr_size=48, us_size=37, r=3, blobs=6, blur=1.5)
    if kind == "3d_r4":
        return synth.case_3d(seed=23, mr_size=48, us_size=40, r=4, blobs=6, blur=1.5,
                             constant_block_frac=0.1)
    if kind == "3d_r5":  # largest radii: 8-row tiles
        return synth.case_3d(seed=24, mr_size=44, us_size=36, r=5, blobs=6, blur=1.5)
    if kind == "3d_r6":
        return synth.case_3d(seed=25, mr_size=44, us_size=36, r=6, blobs=6, blur=1.5)
    if kind == "2dto3d":
        mr = synth.mr_phantom((40, 40, 40), 6, 1.5, seed=31)
        mg = Geometry((40, 40, 40), (1, 1, 1), (0, 0, 0))
        return synth.frame_stack(mr, mg, 1, seed=32, sides=(56,), spacing=0.5, r=3)[0]
    raise KeyError(kind)


def _hr_fixed(case):
    """Same data with the roles of the reference's HighResolutionModality:
    Fixed -- the MR is the fixed grid and the US is warped into it."""
    inv = np.linalg.inv(case.true_mat.astype(np.float64)).astype(np.float32)
    c = synth.Case(case.mode, case.moving_geom, case.moving, case.fixed_geom, case.fixed,
                   list(case.moving_geom.spacing[: (2 if case.mode == "2D" else 3)]), case.r,
                   hr_moving=False, true_params={}, true_mat=inv)
    return c


CASES = ["2d", "2d_r1", "2d_r9", "3d", "3d_r3", "3d_r4", "3d_r5", "3d_r6", "2dto3d"]


@pytest.mark.parametrize("kind", CASES)
def test_fields_and_lc2_match_oracle(kind):
    case = _case(kind)
    ctx = make_context(case)
    mat = case.true_mat
    lc2_gpu, f = ctx.evaluate_fields(mat)
    lc2_ref, of = oracle_eval(case, mat, want_fields=True, use_boxsum=False)
    assert lc2_ref > 0.02
    # warped image and gradient
    mref, gref = of["M"], of["G"]
    assert np.max(np.abs(f["M"] - mref)) <= 2e-5 * max(1.0, np.abs(mref).max())
    assert np.max(np.abs(f["G"] - gref)) <= 2e-5 * max(1.0, np.abs(gref).max())
    # weighting factor
    sref = of["sigma"]
    both = (sref > 0) & (f["sigma"] > 0)
    assert np.array_equal(sref > 0, f["sigma"] > 0)
    assert np.max(np.abs(f["sigma"][both] - sref[both]) / sref[both]) < 1e-5
    # per-voxel measure (absolute, relative to sigma scale)
    assert np.max(np.abs(f["measure"] - of["measure"])) < 2e-4 * sref.max()
    assert abs(lc2_gpu / lc2_ref - 1.0) < REL_LC2, (lc2_gpu, lc2_ref)


@pytest.mark.parametrize("kind", ["2d", "3d", "2dto3d"])
def test_high_res_fixed_mode(kind):
    case = _hr_fixed(_case(kind)) if kind != "2dto3d" else None
    if case is None:
        pytest.skip("2D-to-3D fixes the US frame")
    ctx = make_context(case)
    lc2_gpu = ctx.evaluate(case.true_mat)
    lc2_ref = oracle_eval(case, case.true_mat, use_boxsum=False)
    assert lc2_ref > 0.02
    assert abs(lc2_gpu / lc2_ref - 1.0) < REL_LC2, (lc2_gpu, lc2_ref)


@pytest.mark.parametrize("storage", ["f16", "bf16"])
@pytest.mark.parametrize("kind", ["2d", "3d_r4"])
def test_reduced_storage_matches_oracle_on_rounded_inputs(kind, storage):
    case = _case(kind)
    ctx = make_context(case, storage=storage)
    mats = perturbed(case, np.random.default_rng(5), 3, scale=0.5)
    got = ctx.evaluate_batch(mats)
    for k in range(len(mats)):
        ref = oracle_eval(case, mats[k], storage=storage)
        assert abs(got[k] / ref - 1.0) < REL_LC2, (k, got[k], ref)


@pytest.mark.parametrize("kind", ["2d", "3d", "2dto3d"])
def test_batch_equals_plain_bitwise(kind):
    case = _case(kind)
    ctx = make_context(case, max_batch=3)
    mats = perturbed(case, np.random.default_rng(9), 7)
    batch = ctx.evaluate_batch(mats)
    plain = np.array([ctx.evaluate(m) for m in mats])
    assert np.array_equal(batch, plain)
    again = ctx.evaluate_batch(mats[::-1])[::-1]
    assert np.array_equal(batch, again)


def test_batch_matches_oracle_3d():
    case = _case("3d_r3")
    ctx = make_context(case)
    mats = perturbed(case, np.random.default_rng(3), 5)
    got = ctx.evaluate_batch(mats)
    for k in range(len(mats)):
        ref = oracle_eval(case, mats[k])
        assert abs(got[k] / ref - 1.0) < REL_LC2, (k, got[k], ref)


def test_true_transform_is_best():
    case = _case("2d")
    ctx = make_context(case)
    mats = perturbed(case, np.random.default_rng(1), 16, scale=1.0)
    vals = ctx.evaluate_batch(np.concatenate([case.true_mat[None], mats]))
    assert vals[0] >= vals[1:].max()


def test_out_of_view_transform_gives_zero():
    case = _case("3d")
    ctx = make_context(case)
    far = affine3d((0, 0, 0), (500.0, 0, 0))
    assert ctx.evaluate(far) == 0.0


def test_constant_us_gives_zero():
    case = _case("2d")
    case.fixed = np.full_like(case.fixed, 0.5)
    ctx = make_context(case)
    assert ctx.evaluate(case.true_mat) == 0.0


def test_exact_linear_us_gives_one():
    """US = 0.7 M + 0.5 G + 0.05 on the identity transform: LC2 == 1 up to the
    FP32 Sobel of the device."""
    case = _case("2d")
    from oracle import oracle as O
    m = case.moving.astype(np.float64)
    g = O.sobel(2, (64, 64, 1), m.ravel()).reshape(m.shape)
    case.fixed = (0.7 * m + 0.5 * g + 0.05).astype(np.float32)
    ctx = make_context(case)
    v = ctx.evaluate(np.eye(3, dtype=np.float32))
    assert abs(v - 1.0) < 1e-5


def test_nan_input_rejected():
    case = _case("2d")
    ctx = capi.Context(case.mode, case.fixed_geom, case.moving_geom, case.virt_spacing, case.r)
    bad = case.fixed.copy()
    bad[3, 3] = np.nan
    with pytest.raises(capi.LC2Error) as e:
        ctx.set_images(bad, case.moving)
    assert e.value.status == 1
    with pytest.raises(capi.LC2Error) as e:
        ctx.evaluate(np.eye(3, dtype=np.float32))
    assert e.value.status == 4  # images never set


def test_odd_sizes_and_tiny_grids():
    rng = np.random.default_rng(17)
    for (nx, ny, nz, r) in [(7, 5, 3, 1), (33, 9, 11, 2), (65, 17, 1, 4)]:
        mode = "3D" if nz > 1 else "2D"
        g = Geometry((nx, ny, nz), (1, 1, 1), (0, 0, 0))
        mov = rng.random((nz, ny, nx)).astype(np.float32)
        fix = (rng.random((nz, ny, nx)) + 0.2).astype(np.float32)
        vs = [1.0, 1.0, 1.0][: (3 if mode == "3D" else 2)]
        case = synth.Case(mode, g, fix, g, mov, vs, r, True, {}, None)
        mat = np.eye(4 if mode == "3D" else 3, dtype=np.float32)
        mat[0, -1] = 0.37
        ctx = make_context(case)
        got = ctx.evaluate(mat)
        ref = oracle_eval(case, mat, use_boxsum=False)
        if ref == 0.0:
            assert got == 0.0
        else:
            assert abs(got / ref - 1.0) < REL_LC2, (nx, ny, nz, r, got, ref)


@pytest.mark.parametrize("name", ["2d_r3", "2d_r1", "3d_r2", "3d_r3", "3d_r4", "2dto3d_r3",
                                  "2d_hrfixed_r2"])
def test_fields_match_reference_kernels(name):
    """The CUDA path against the reference's own kernels (golden fixtures):
    resampled images, Sobel magnitude and weighting factor to FP32 accuracy,
    weighted similarity on every patch where the reference's CG converged."""
    from tests.test_golden import load_case

    mode, fg, fixed, mg, moving, vs, r, hrm, mat, ref = load_case(name)
    G = lambda g: Geometry(tuple(g.dim), tuple(g.spacing), tuple(g.origin))
    ctx = capi.Context(mode, G(fg), G(mg), vs, r, hrm)
    ctx.set_images(fixed, moving)
    lc2, f = ctx.evaluate_fields(mat)
    for k in "UM":
        assert np.max(np.abs(f[k] - ref[k])) <= 2e-5 * max(1.0, np.abs(ref[k]).max()), k
    assert np.max(np.abs(f["G"] - ref["G"])) <= 2e-5 * max(1.0, np.abs(ref["G"]).max())
    w = ref["W"].astype(np.float64)
    assert np.array_equal(w > 0, f["sigma"] > 0)
    both = w > 0
    assert np.max(np.abs(f["sigma"][both] - w[both]) / w[both]) < 2e-5
    S = ref["S"].astype(np.float64)
    close = np.abs(S - f["measure"]) <= 1e-4 * np.maximum(w, 1e-12)
    assert close[both].mean() > 0.975


@pytest.mark.parametrize("kind", ["2d", "3d"])
def test_degenerate_inputs(kind):
    """Edge cases with known answers: a constant ultrasound has no valid
    patch (every sigma is 0, LC2 = 0/0 -> 0), and a transform that maps the
    whole virtual grid outside the moving image leaves M = G = 0 (no measure,
    LC2 = 0), on the GPU as in the oracle."""
    case = _case(kind)
    flat = synth.Case(case.mode, case.fixed_geom, np.full_like(case.fixed, 0.7),
                      case.moving_geom, case.moving, case.virt_spacing, case.r, case.hr_moving,
                      case.true_params, case.true_mat)
    ctx = make_context(flat)
    assert ctx.evaluate(flat.true_mat) == 0.0
    assert oracle_eval(flat, flat.true_mat) == 0.0
    away = case.true_mat.copy()
    away[0, -1] += 1e4  # translate far outside the moving image
    ctx2 = make_context(case)
    assert ctx2.evaluate(away) == 0.0
    assert oracle_eval(case, away) == 0.0
    np.testing.assert_array_equal(ctx2.evaluate_batch(np.stack([away, away])), [0.0, 0.0])


@pytest.mark.parametrize("hr_moving", [True, False])
@pytest.mark.parametrize("kind", ["2d", "3d"])
def test_flat_mr_gives_zero(kind, hr_moving):
    """A flat MR under the identity, with the ultrasound zero (invalid) in a
    border band wider than r + 1: every valid patch lies where M is constant
    and G = 0 (the zero-padded border, where the Sobel sees an edge, only
    enters invalid patches), so no regressor has variance, every measure is
    clipped to 0 and LC2 = 0 while sigma > 0 -- on the GPU as in the oracle."""
    from lc2registration_gb300.geometry import Geometry

    nd = 2 if kind == "2d" else 3
    dims = (48, 40, 1) if nd == 2 else (40, 36, 32)
    r = 3 if nd == 2 else 2
    g = Geometry(dims, (1, 1, 1), (0, 0, 0))
    rng = np.random.default_rng(31)
    shape = dims[::-1] if nd == 3 else dims[1::-1]
    us = (rng.random(shape) * 0.5 + 0.2).astype(np.float32)
    b = r + 2
    band = np.ones(shape, dtype=bool)
    band[tuple(slice(b, n - b) for n in shape)] = False
    us[band] = 0.0
    mr = np.full(shape, 0.6, dtype=np.float32)
    mode = "2D" if nd == 2 else "3D"
    ident = np.eye(nd + 1, dtype=np.float32)
    if hr_moving:
        case = synth.Case(mode, g, us, g, mr, [1.0] * nd, r, True, {}, ident)
    else:
        case = synth.Case(mode, g, mr, g, us, [1.0] * nd, r, False, {}, ident)
    ctx = make_context(case)
    assert ctx.evaluate(ident) == 0.0
    assert oracle_eval(case, ident, use_boxsum=False) == 0.0
    # sigma is not zero everywhere: the zero comes from the clipped measures
    _, f = ctx.evaluate_fields(ident)
    assert f["sigma"].max() > 0.0 and f["measure"].max() == 0.0


@pytest.mark.parametrize("hr_moving", [True, False])
@pytest.mark.parametrize("kind", ["2d", "3d_r3"])
def test_extreme_transforms_match_oracle(kind, hr_moving):
    """Large rotations (about 30, 90 and 180 degrees), strong scaling (0.6x,
    1.7x), shear and a translation that leaves part of the grid out of view:
    the sampler's interior fast path must switch off exactly where samples
    leave the moving image, and the values follow the oracle.

    The angles sit off exact multiples of 90 degrees: there every sample
    lands on an integer pixel and the border ones exactly on 0 or dim - 1,
    where inside/outside flips on a 1e-7-voxel difference (the float32
    matrix's cos 90 = -4.4e-8) -- below the sampler's FP32 resolution, so
    the FP64 oracle and any FP32 evaluation, the reference's included, may
    decide such ties differently."""
    from lc2registration_gb300.geometry import affine2d, affine3d

    case = _case(kind)
    if not hr_moving:
        case = _hr_fixed(case)
    c = case.fixed_geom.center()
    if case.mode == "2D":
        mats = [affine2d(a, t, s, sh, c[:2], (0, 0)) for a, t, s, sh in
                [(30.0, (2, -3), (1.0, 1.0), 0.0), (90.4, (0.3, 0), (1.0, 1.0), 0.0),
                 (179.3, (1, 1), (1.0, 1.0), 0.0), (10.0, (0, 0), (0.6, 0.6), 0.0),
                 (-15.0, (5, 0), (1.7, 1.2), 0.2), (5.0, (20, -15), (1.0, 1.0), 0.0)]]
    else:
        mats = [affine3d(rot, t, s, sh, c, (0, 0, 0)) for rot, t, s, sh in
                [((30.0, 0, 0), (2, -3, 1), (1, 1, 1), (0, 0, 0)),
                 ((0, 90.4, 0), (0.3, 0, 0), (1, 1, 1), (0, 0, 0)),
                 ((0, 0, 179.3), (1, 1, 0), (1, 1, 1), (0, 0, 0)),
                 ((10.0, -20.0, 15.0), (0, 0, 0), (0.6, 0.7, 0.6), (0.1, 0, -0.1)),
                 ((5.0, 5.0, 5.0), (12, -10, 8), (1.7, 1.3, 1.0), (0, 0.2, 0))]]
    mats = np.stack(mats).astype(np.float32)
    ctx = make_context(case)
    got = ctx.evaluate_batch(mats)
    for k in range(len(mats)):
        ref = oracle_eval(case, mats[k], use_boxsum=False)
        if ref == 0.0:
            assert got[k] == 0.0, k
        else:
            assert abs(got[k] / ref - 1.0) < REL_LC2, (k, got[k], ref)
