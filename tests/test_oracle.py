"""CPU tests of the FP64 oracle: internal consistency and known answers.

The reference has no tests or golden LC2 values; the oracle is pinned by
(a) the reference's own transform builders run here (test_golden.py),
(b) the known-answer cases below, derived from the reference's formulas
(src/cu_LC2/cu_lc2_2d.cu:88-480, cu_lc2_3d.cu:181-618), and
(c) two independent oracle paths (direct per-patch two-pass vs separable
box sums) that must agree.
"""
import numpy as np
import pytest

from oracle import oracle as O


def _rand_case(rng, nd, dim, lo=0.1):
    n = int(np.prod(dim))
    U = rng.random(n) + lo
    M = rng.random(n)
    G = O.sobel(nd, dim, M)
    return U, M, G


@pytest.mark.parametrize("nd,dim,r", [(2, (17, 13, 1), 1), (2, (21, 19, 1), 3), (2, (30, 9, 1), 4),
                                      (3, (11, 9, 7), 1), (3, (12, 11, 10), 2), (3, (13, 14, 12), 3)])
def test_direct_matches_boxsum(nd, dim, r):
    rng = np.random.default_rng(nd * 100 + r)
    U, M, G = _rand_case(rng, nd, dim)
    s = O.sigma(nd, dim, r, U)
    m = O.measure_direct(nd, dim, r, U, M, G, s)
    sm, ss, mb = O.lc2_boxsum(nd, dim, r, U, M, G)
    assert np.allclose(mb, m, rtol=1e-9, atol=1e-12)
    assert abs(sm - m.sum()) <= 1e-9 * max(1.0, abs(sm))
    assert abs(ss - s.sum()) <= 1e-9 * max(1.0, abs(ss))


@pytest.mark.parametrize("nd,dim,r", [(2, (23, 17, 1), 2), (3, (12, 13, 11), 2)])
def test_exact_linear_model_gives_one(nd, dim, r):
    """U = a M + b G + c exactly: every valid patch fits with zero residual,
    so measure == sigma and LC2 == 1."""
    rng = np.random.default_rng(7)
    M = rng.random(int(np.prod(dim)))
    G = O.sobel(nd, dim, M)
    U = 0.7 * M + 0.5 * G + 0.05
    s = O.sigma(nd, dim, r, U)
    m = O.measure_direct(nd, dim, r, U, M, G, s)
    assert (s > 0).sum() > 0
    assert abs(m.sum() / s.sum() - 1.0) < 1e-12


def test_constant_us_gives_zero_sigma():
    """Zero variance: sigma = 0 everywhere, sum(sigma) = 0, LC2 -> 0
    (NaN/Inf -> 0, cu_lc2_3d.cu:1189-1191)."""
    dim = (16, 15, 1)
    U = np.full(int(np.prod(dim)), 0.5)
    M = np.random.default_rng(3).random(U.size)
    G = O.sobel(2, dim, M)
    s = O.sigma(2, dim, 2, U)
    assert s.max() == 0.0
    sm, ss, _ = O.lc2_boxsum(2, dim, 2, U, M, G)
    assert sm == 0.0 and ss == 0.0


def test_flat_mr_gives_zero_measure():
    """A constant high-resolution image explains nothing: every measure 0."""
    dim = (14, 13, 1)
    rng = np.random.default_rng(4)
    U = rng.random(int(np.prod(dim))) + 0.2
    M = np.full(U.size, 0.3)
    G = np.zeros(U.size)
    s = O.sigma(2, dim, 2, U)
    m = O.measure_direct(2, dim, 2, U, M, G, s)
    assert s.max() > 0 and m.max() == 0.0


def test_sigma_validity_rules():
    """A single value <= 1e-6 invalidates every patch containing it; patches
    touching the border are invalid (zero padding)."""
    dim = (20, 20, 1)
    rng = np.random.default_rng(5)
    U = rng.random(400) + 0.1
    U[10 * 20 + 10] = 1e-6  # not > 1e-6
    s = O.sigma(2, dim, 2, U).reshape(20, 20)
    assert s[8:13, 8:13].max() == 0.0
    assert s[:2].max() == 0.0 and s[-2:].max() == 0.0 and s[:, :2].max() == 0.0
    assert s[5, 5] > 0.0


def test_variance_threshold():
    """Sample variance <= 1e-6 gives sigma = 0 (cu_lc2_2d.cu:167-173)."""
    dim = (12, 12, 1)
    base = np.full(144, 0.5)
    base[::2] += 1.5e-3  # variance ~ 5.6e-7 < 1e-6
    s = O.sigma(2, dim, 1, base)
    assert s.max() == 0.0
    base2 = np.full(144, 0.5)
    base2[::2] += 3e-3  # variance ~ 2.25e-6 > 1e-6
    assert O.sigma(2, dim, 1, base2).max() > 0.0


def test_sobel_matches_numpy():
    rng = np.random.default_rng(6)
    a = rng.random((5, 6, 7))  # z, y, x
    g = O.sobel(3, (7, 6, 5), a.ravel()).reshape(5, 6, 7)
    p = np.pad(a, 1)
    h, hp = np.array([1.0, 2.0, 1.0]), np.array([-1.0, 0.0, 1.0])
    gx = np.zeros_like(a); gy = np.zeros_like(a); gz = np.zeros_like(a)
    for k in range(3):
        for j in range(3):
            for i in range(3):
                v = p[k:k + 5, j:j + 6, i:i + 7]
                gx += hp[i] * h[j] * h[k] * v
                gy += h[i] * hp[j] * h[k] * v
                gz += h[i] * h[j] * hp[k] * v
    assert np.allclose(g, np.sqrt(gx ** 2 + gy ** 2 + gz ** 2), rtol=1e-13, atol=1e-13)


def test_resample_identity_and_bounds():
    """Identity transform on aligned grids reproduces the image, including the
    last row/column (inclusive [0, dim-1] bound); a shift of half a voxel
    gives the mean of neighbours; samples beyond the edge are 0."""
    rng = np.random.default_rng(8)
    img = rng.random((6, 9)).astype(np.float32)
    g = O.Geom((9, 6, 1), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0))
    ident = np.eye(3, dtype=np.float32)
    out = O.resample(2, g, g, img, ident).reshape(6, 9)
    assert np.array_equal(out, img.astype(np.float64))
    sh = ident.copy(); sh[0, 2] = 0.5
    out = O.resample(2, g, g, img, sh).reshape(6, 9)
    assert np.allclose(out[:, :8], 0.5 * (img[:, :8].astype(np.float64) + img[:, 1:]))
    assert np.all(out[:, 8] == 0.0)


def test_virtual_geometry_matches_reference_formula():
    g = O.Geom((321, 297, 1), (0.50838, 0.50838, 1.0), (0.0, 0.0, 0.0))
    v = O.virtual_geom(2, g, (1.0, 1.0))
    assert v.dim[:2] == [164, 151]  # config/Data/fixed.bin is 164 x 151
    v = O.virtual_geom(2, g, (0.9, 0.9))
    assert v.dim[:2] == [182, 168]  # *_virtual.bin is 182 x 168


def test_nmi_known_values():
    rng = np.random.default_rng(0)
    U = rng.random(4000).astype(np.float32)
    assert abs(O.nmi(U, U) - 2.0) < 1e-12           # identical images
    assert abs(O.nmi(U, 3 * U + 1) - 2.0) < 1e-12   # affine intensity map, same bins
    c = np.full(4000, 0.5, dtype=np.float32)
    assert O.nmi(U, c) == 1.0                        # constant image: H = 0, H(U,M) = H(U)
    V = rng.random(4000).astype(np.float32)
    assert 1.0 < O.nmi(U, V) < O.nmi(U, 0.5 * U + 0.1 * V)
