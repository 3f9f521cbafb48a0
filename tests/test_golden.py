"""Pins the transform math against the reference's own code.

tests/golden/ref_mappers.txt was produced by running the reference's
Spatial3DMapper::AffineInit / GetMyselfInversed and Spatial2DMapper::AffineInit
(src/Interpolator/spatialMappers.cuh:315-433, :637-850, :999-1033), compiled
from the reference sources by oracle/Makefile target `ref`
(tests/golden/make_golden.py). The oracle's, the Python helper's and the C
library's builders must reproduce those matrices. The reference builds them
in float32 (from double sin/cos); ours round once from double, so the
comparison allows a few float32 ulps of the largest term.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from lc2registration_gb300 import capi, geometry

HERE = os.path.dirname(os.path.abspath(__file__))


def _cases():
    a3, a2 = [], []
    with open(os.path.join(HERE, "golden", "ref_mappers.txt")) as f:
        for line in f:
            parts = line.split("|")
            head = parts[0].split()
            vals = [float(v) for v in head[1:]]
            if head[0] == "A3":
                a3.append((vals, [float(v) for v in parts[1].split()], [float(v) for v in parts[2].split()]))
            else:
                a2.append((vals, [float(v) for v in parts[1].split()]))
    return a3, a2


A3, A2 = _cases()


def _close(got, ref, rel=2e-6):
    got = np.asarray(got, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    scale = np.maximum(1.0, np.abs(ref))
    return np.all(np.abs(got - ref) <= rel * 64 * scale), np.max(np.abs(got - ref) / scale)


def test_fixture_present():
    assert len(A3) == 24 and len(A2) == 24


@pytest.mark.parametrize("i", range(24))
def test_affine3d_matches_reference(i):
    v, ref, _ = A3[i]
    rot, tr, sc, sh, c, f = v[0:3], v[3:6], v[6:9], v[9:12], v[12:15], v[15:18]
    for got in (O.affine3d(rot, tr, sc, sh, c, f), geometry.affine3d(rot, tr, sc, sh, c, f),
                capi.affine_3d(rot, tr, sc, sh, c, f)):
        ok, err = _close(got, ref)
        assert ok, err


@pytest.mark.parametrize("i", range(24))
def test_affine2d_matches_reference(i):
    v, ref = A2[i]
    r, tr, sc, sh, c, f = v[0], v[1:3], v[3:5], v[5], v[6:8], v[8:10]
    for got in (O.affine2d(r, tr, sc, sh, c, f), geometry.affine2d(r, tr, sc, sh, c, f),
                capi.affine_2d(r, tr, sc, sh, c, f)):
        ok, err = _close(got, ref)
        assert ok, err


@pytest.mark.parametrize("i", range(24))
def test_inverse_matches_reference(i):
    _, mat, inv = A3[i]
    got = capi.invert_affine_3d(np.array(mat, dtype=np.float32))
    ok, err = _close(got, inv, rel=2e-5)
    assert ok, err


# ---------------------------------------------------------------------------
# The reference's own LC2 kernels (run on the CPU under
# oracle/ref_golden/kernel_emu.cpp) on seeded inputs: ref_lc2_cases.npz.
# ---------------------------------------------------------------------------

def _lc2_cases():
    d = np.load(os.path.join(HERE, "golden", "ref_lc2_cases.npz"))
    names = sorted({k.split("/")[0] for k in d.files})
    return d, names


_D, _NAMES = _lc2_cases()


def load_case(name):
    """(mode, fixed_geom, fixed, moving_geom, moving, vspacing, r, hr_moving, mat, ref fields)."""
    g = _D[f"{name}/geom"]
    meta = _D[f"{name}/meta"]
    mode = {0: "2D", 1: "3D", 2: "2DTo3D"}[int(meta[3])]
    geo = [O.Geom([int(v) for v in row[0:3]], list(row[3:6]), list(row[6:9])) for row in g]
    nd = 2 if mode == "2D" else 3
    vs = list(_D[f"{name}/vspacing"][:nd])
    ref = {k: _D[f"{name}/{k}"] for k in "UMGWS"}
    return (mode, geo[0], _D[f"{name}/fixed"], geo[1], _D[f"{name}/moving"], vs, int(meta[1]),
            bool(meta[2]), _D[f"{name}/mat"], ref)


@pytest.mark.parametrize("name", _NAMES)
def test_oracle_matches_reference_kernels(name):
    mode, fg, fixed, mg, moving, vs, r, hrm, mat, ref = load_case(name)
    lc2, f = O.lc2_eval(mode, fg, fixed, mg, moving, vs, r, mat, hr_moving=hrm, use_boxsum=False,
                        want_fields=True)
    # resampling, Sobel and the weighting factor are deterministic FP32 in the
    # reference: they agree with the FP64 oracle to FP32 rounding
    for k, ok in (("U", "U"), ("M", "M")):
        assert np.max(np.abs(ref[k] - f[ok])) <= 2e-6 * max(1.0, np.abs(f[ok]).max()), k
    assert np.max(np.abs(ref["G"] - f["G"])) <= 1e-5 * max(1.0, np.abs(f["G"]).max())
    w, s = ref["W"].astype(np.float64), f["sigma"]
    assert np.array_equal(w > 0, s > 0)
    both = s > 0
    assert np.max(np.abs(w[both] - s[both]) / s[both]) < 2e-5
    # weighted similarity: the reference solves each patch by FP32 conjugate
    # gradient from x = 0 (stop at |g| < 1e-6 in 2D, 1e-4 in 3D, at most 20
    # iterations). Most patches reach the exact LS fit; a few stop short or end
    # in 0/0 -> NaN -> 0 (2D r=1: ~2% of patches). The oracle keeps the exact
    # fit, so the comparison is on the converged patches, and the others may
    # only have lost fit, never gained it.
    S, m = ref["S"].astype(np.float64), f["measure"]
    close = np.abs(S - m) <= 1e-4 * np.maximum(s, 1e-12)
    frac = close[both].mean()
    assert frac > 0.975, frac
    bad = ~close & both
    assert np.all(S[bad] <= m[bad] + 1e-6 * s[bad])
    # LC2 over the converged patches agrees to the CG stopping accuracy
    lc2_ref = S[close].sum() / w.sum()
    lc2_orc = m[close].sum() / s.sum()
    assert abs(lc2_ref / lc2_orc - 1.0) < 2e-5
