"""ctypes binding of oracle/_ref/libref_kernels.so: the reference's own LC2
kernels run on the CPU by oracle/ref_golden/kernel_emu.cpp (test
infrastructure; needs the reference sources to build, so it exists only where
`make -C oracle ref` ran)."""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(_HERE, "_ref", "libref_kernels.so")


def available() -> bool:
    return os.path.exists(LIB)


def _arr(v, t):
    return np.ascontiguousarray(v, dtype=t)


def evaluate(mode, fixed_geom, fixed, moving_geom, moving, virt_geom, mat, r, hr_moving=True):
    """Runs the reference's resample + Sobel + weighting + CG-similarity
    kernels. Returns dict of float32 fields U, M, G, W (weighting factor),
    S (weighted similarity) on the virtual grid."""
    lib = ctypes.CDLL(LIB)
    fp, ip = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int)
    n = int(np.prod(virt_geom.dim))
    out = {k: np.zeros(n, dtype=np.float32) for k in "UMGWS"}
    keep = []

    def g(geom):
        d = _arr(list(geom.dim), np.int32)
        s = _arr(list(geom.spacing), np.float32)
        o = _arr(list(geom.origin), np.float32)
        keep.extend([d, s, o])
        return [d.ctypes.data_as(ip), s.ctypes.data_as(fp), o.ctypes.data_as(fp)]

    f = _arr(fixed, np.float32).ravel()
    m = _arr(moving, np.float32).ravel()
    mt = _arr(mat, np.float32).ravel()
    args = g(fixed_geom) + [f.ctypes.data_as(fp)] + g(moving_geom) + [m.ctypes.data_as(fp)] + \
        g(virt_geom) + [mt.ctypes.data_as(fp), ctypes.c_int(int(hr_moving)), ctypes.c_int(int(r))]
    outs = [out[k].ctypes.data_as(fp) for k in "UMGWS"]
    if mode == "2D":
        lib.ref_eval_2d(*args, *outs)
    else:
        lc2_nd = 3 if mode == "3D" else 2
        lib.ref_eval_3d(*args, ctypes.c_int(lc2_nd), *outs)
    return out
