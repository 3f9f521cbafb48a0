"""CPU checks of the C ABI library: it builds, loads, exports every symbol
include/lc2.h declares, and rejects bad arguments before touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from lc2registration_gb300 import capi
from lc2registration_gb300.geometry import Geometry

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(lc2_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_library_loads_and_exports_all_declared_symbols():
    lib = capi.load()
    declared = _declared()
    assert declared, "no declarations found"
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing
    assert set(declared) == set(capi.EXPORTED)


def test_version_and_error_string():
    lib = capi.load()
    assert b"sm_103a" in lib.lc2_version()
    assert isinstance(lib.lc2_last_error(), bytes)


def test_rejects_bad_config_without_gpu():
    g = Geometry((32, 32, 1), (1, 1, 1), (0, 0, 0))
    with pytest.raises(capi.LC2Error) as e:
        capi.Context("2D", g, g, (1.0, 1.0), patch_size=0)
    assert e.value.status == 6  # unsupported patch size
    with pytest.raises(capi.LC2Error) as e:
        capi.Context("3D", Geometry((8, 8, 8), (1, 1, 1), (0, 0, 0)), g, (1, 1, 1), patch_size=7)
    assert e.value.status == 6
    bad = Geometry((32, 32, 1), (0.0, 1, 1), (0, 0, 0))
    with pytest.raises(capi.LC2Error) as e:
        capi.Context("2D", bad, g, (1.0, 1.0), patch_size=3)
    assert e.value.status == 1
    lib = capi.load()
    h = ctypes.c_void_p()
    assert lib.lc2_create(None, ctypes.byref(h)) == 1


@pytest.mark.parametrize("spacing", [1e-6, 0.001])
def test_rejects_oversized_virtual_grid_without_gpu(spacing):
    """A resampled spacing that would make the virtual grid overflow the
    kernels' 32-bit slice indices or the 65535-tile grid limit is refused on
    the host (status 6), before any device allocation."""
    g = Geometry((512, 512, 1), (1, 1, 1), (0, 0, 0))
    with pytest.raises(capi.LC2Error) as e:
        capi.Context("2D", g, g, (spacing, spacing), patch_size=3)
    assert e.value.status == 6
    assert "virtual" in str(e.value)


def test_singular_inverse_rejected():
    with pytest.raises(capi.LC2Error) as e:
        capi.invert_affine_3d(np.zeros((4, 4), dtype=np.float32))
    assert e.value.status == 5


def test_null_context_calls_fail_cleanly():
    lib = capi.load()
    out = ctypes.c_double()
    m = (ctypes.c_float * 16)()
    assert lib.lc2_evaluate(None, m, ctypes.byref(out)) != 0
    assert lib.lc2_destroy(None) == 0


def test_stack_rejects_bad_arguments_without_gpu():
    lib = capi.load()
    h = ctypes.c_void_p()
    g = capi._geom(Geometry((16, 16, 16), (1, 1, 1), (0, 0, 0)))
    assert lib.lc2_stack_create(None, 3, 0, 0, ctypes.byref(h)) == 1
    assert lib.lc2_stack_create(ctypes.byref(g), 0, 0, 0, ctypes.byref(h)) == 6
    assert lib.lc2_stack_create(ctypes.byref(g), 13, 0, 0, ctypes.byref(h)) == 6
    assert lib.lc2_stack_create(ctypes.byref(g), 3, 7, 0, ctypes.byref(h)) == 1
    bad = capi._geom(Geometry((16, 16, 16), (1, -1, 1), (0, 0, 0)))
    assert lib.lc2_stack_create(ctypes.byref(bad), 3, 0, 0, ctypes.byref(h)) == 1
    assert lib.lc2_stack_evaluate(None, 1, None, None, None) == 1
    assert lib.lc2_stack_frames(None) == 0
    assert lib.lc2_stack_destroy(None) == 0


def test_noalloc_rejects_wrapping_sizes_without_gpu():
    """lc2_evaluate_noalloc bounds the virtual grid axis by axis, so a grid
    whose voxel count would wrap a 64-bit product (2^30 x 2^30 x 16) is
    refused like any grid over LC2_NOALLOC_MAX_VOXELS, and so is a moving
    image beyond 32-bit gather indices -- both before any device call."""
    lib = capi.load()
    dummy = ctypes.c_void_p(256)  # never dereferenced: the call fails first
    m = (ctypes.c_float * 16)(*np.eye(4, dtype=np.float32).ravel())

    def call(vdim, mdim):
        v = capi._geom(Geometry(vdim, (1, 1, 1), (0, 0, 0)))
        g = capi._geom(Geometry(mdim, (1, 1, 1), (0, 0, 0)))
        return lib.lc2_evaluate_noalloc(1, ctypes.byref(v), ctypes.byref(g), 2, dummy, dummy, m,
                                        dummy, None)

    assert call((1 << 30, 1 << 30, 16), (8, 8, 8)) == 6
    assert b"LC2_NOALLOC_MAX_VOXELS" in lib.lc2_last_error()
    assert call((1 << 10, 1 << 10, 2), (8, 8, 8)) == 6
    assert call((16, 16, 16), (65536, 65536, 2)) == 6
    assert b"2^31" in lib.lc2_last_error()
