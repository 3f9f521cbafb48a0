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
