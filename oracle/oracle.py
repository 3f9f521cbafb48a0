"""ctypes binding of the FP64 LC2 oracle (test infrastructure only).

The oracle is the checker for the CUDA path. Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline/reference legs
import this module. The product library never calls it.

The C sources (``lc2_oracle.c``) restate, in IEEE double, the reference's
resampling (src/Interpolator/interpolator.cu:69-232), Sobel
(src/cu_LC2/cu_lc2_2d.cu:25-86, cu_lc2_3d.cu:100-179), weighting factor
(cu_lc2_2d.cu:88-180, cu_lc2_3d.cu:181-287), per-patch least-squares measure
(cu_lc2_2d.cu:182-480, cu_lc2_3d.cu:289-618) and ratio reduction
(cu_lc2_2d.cu:599-653, cu_lc2_3d.cu:1119-1194).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liblc2oracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle shared library with the committed Makefile."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "lc2_oracle.c"))
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class _Geom(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int * 3),
        ("spacing", ctypes.c_float * 3),
        ("origin", ctypes.c_float * 3),
    ]


@dataclass
class Geom:
    """Image/volume geometry: dims (x, y, z), spacing and origin in mm."""

    dim: Sequence[int]
    spacing: Sequence[float]
    origin: Sequence[float]

    def c(self) -> _Geom:
        g = _Geom()
        d = list(self.dim) + [1] * (3 - len(self.dim))
        s = list(self.spacing) + [1.0] * (3 - len(self.spacing))
        o = list(self.origin) + [0.0] * (3 - len(self.origin))
        for a in range(3):
            g.dim[a] = int(d[a])
            g.spacing[a] = float(s[a])
            g.origin[a] = float(o[a])
        return g

    @property
    def n(self) -> int:
        d = list(self.dim) + [1] * (3 - len(self.dim))
        return int(d[0] * d[1] * d[2])


_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)


def _load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = ctypes.CDLL(_LIB_PATH)
    gp = ctypes.POINTER(_Geom)
    lib.or_resample.argtypes = [ctypes.c_int, gp, gp, _fp, _fp, _dp]
    lib.or_sobel.argtypes = [ctypes.c_int, _ip, _dp, _dp]
    lib.or_sigma.argtypes = [ctypes.c_int, _ip, ctypes.c_int, _dp, _dp]
    lib.or_measure_direct.argtypes = [ctypes.c_int, _ip, ctypes.c_int, _dp, _dp, _dp, _dp, _dp]
    lib.or_lc2_boxsum.argtypes = [ctypes.c_int, _ip, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp,
                                  ctypes.c_int]
    lib.or_lc2_eval.restype = ctypes.c_double
    lib.or_lc2_eval.argtypes = [ctypes.c_int, ctypes.c_int, gp, _fp, gp, _fp, _fp, ctypes.c_int,
                                ctypes.c_int, _fp, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp,
                                _dp, _dp, _dp]
    lib.or_virtual_geom.argtypes = [ctypes.c_int, gp, _fp, gp]
    lib.or_affine3d.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, _fp]
    lib.or_nmi.restype = ctypes.c_double
    lib.or_nmi.argtypes = [_fp, _fp, ctypes.c_longlong]
    lib.or_affine2d.argtypes = [ctypes.c_double, _dp, _dp, ctypes.c_double, _dp, _dp, _fp]
    _lib = lib
    return lib


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def _dims3(shape_xyz: Sequence[int]) -> np.ndarray:
    d = list(shape_xyz) + [1] * (3 - len(shape_xyz))
    return np.array(d[:3], dtype=np.int32)


def virtual_geom(ndim: int, fixed: Geom, virt_spacing: Sequence[float]) -> Geom:
    lib = _load()
    out = _Geom()
    sv = _f32(list(virt_spacing) + [1.0] * (3 - len(virt_spacing)))
    fg = fixed.c()
    lib.or_virtual_geom(ndim, ctypes.byref(fg), _ptr(sv, _fp), ctypes.byref(out))
    return Geom(list(out.dim), list(out.spacing), list(out.origin))


def resample(ndim: int, virt: Geom, src_geom: Geom, src: np.ndarray, mat) -> np.ndarray:
    lib = _load()
    src = _f32(src)
    m = _f32(mat).ravel()
    out = np.empty(virt.n, dtype=np.float64)
    vg, sg = virt.c(), src_geom.c()
    lib.or_resample(ndim, ctypes.byref(vg), ctypes.byref(sg), _ptr(src, _fp), _ptr(m, _fp),
                    _ptr(out, _dp))
    return out


def sobel(ndim: int, dim_xyz: Sequence[int], a: np.ndarray) -> np.ndarray:
    lib = _load()
    a = _f64(a).ravel()
    out = np.empty_like(a)
    d = _dims3(dim_xyz)
    lib.or_sobel(ndim, _ptr(d, _ip), _ptr(a, _dp), _ptr(out, _dp))
    return out


def sigma(ndim: int, dim_xyz: Sequence[int], r: int, U: np.ndarray) -> np.ndarray:
    lib = _load()
    U = _f64(U).ravel()
    out = np.empty_like(U)
    d = _dims3(dim_xyz)
    lib.or_sigma(ndim, _ptr(d, _ip), r, _ptr(U, _dp), _ptr(out, _dp))
    return out


def measure_direct(ndim, dim_xyz, r, U, M, G, sig) -> np.ndarray:
    lib = _load()
    U, M, G, sig = (_f64(a).ravel() for a in (U, M, G, sig))
    out = np.empty_like(U)
    d = _dims3(dim_xyz)
    lib.or_measure_direct(ndim, _ptr(d, _ip), r, _ptr(U, _dp), _ptr(M, _dp), _ptr(G, _dp),
                          _ptr(sig, _dp), _ptr(out, _dp))
    return out


def lc2_boxsum(ndim, dim_xyz, r, U, M, G, sig=None, nthreads: int = 0):
    """Returns (sum_measure, sum_sigma, measure array)."""
    lib = _load()
    U, M, G = (_f64(a).ravel() for a in (U, M, G))
    meas = np.empty_like(U)
    sums = np.zeros(2, dtype=np.float64)
    d = _dims3(dim_xyz)
    sp = _ptr(_f64(sig).ravel(), _dp) if sig is not None else None
    keep = _f64(sig).ravel() if sig is not None else None
    if keep is not None:
        sp = _ptr(keep, _dp)
    lib.or_lc2_boxsum(ndim, _ptr(d, _ip), r, _ptr(U, _dp), _ptr(M, _dp), _ptr(G, _dp), sp,
                      _ptr(meas, _dp), _ptr(sums, _dp), nthreads)
    return float(sums[0]), float(sums[1]), meas


def lc2_eval(mode: str, fixed_geom: Geom, fixed: np.ndarray, moving_geom: Geom,
             moving: np.ndarray, virt_spacing: Sequence[float], r: int, mat,
             hr_moving: bool = True, use_boxsum: bool = True, nthreads: int = 0,
             want_fields: bool = False):
    """Full FP64 LC2 evaluation.

    mode: "2D", "3D" or "2DTo3D" (the three registration modes of the
    reference CLI, src/mainRegistrationTool/main.cu:728-827). ``mat`` is the
    row-major virtual->moving mm matrix (3x3 for 2D, 4x4 otherwise).
    Returns lc2, or (lc2, fields) with fields = dict(U, M, G, sigma, measure,
    sums) when want_fields.
    """
    lib = _load()
    rs_nd, lc_nd = {"2D": (2, 2), "3D": (3, 3), "2DTo3D": (3, 2)}[mode]
    fixed, moving = _f32(fixed).ravel(), _f32(moving).ravel()
    m = _f32(mat).ravel()
    sv = _f32(list(virt_spacing) + [1.0] * (3 - len(virt_spacing)))
    vg = virtual_geom(rs_nd, fixed_geom, virt_spacing)
    N = vg.n
    outs = [np.empty(N, dtype=np.float64) for _ in range(5)] if want_fields else [None] * 5
    sums = np.zeros(2, dtype=np.float64)
    fg, mg = fixed_geom.c(), moving_geom.c()
    ptrs = [(_ptr(o, _dp) if o is not None else None) for o in outs]
    val = lib.or_lc2_eval(rs_nd, lc_nd, ctypes.byref(fg), _ptr(fixed, _fp), ctypes.byref(mg),
                          _ptr(moving, _fp), _ptr(sv, _fp), int(r), int(bool(hr_moving)),
                          _ptr(m, _fp), int(bool(use_boxsum)), int(nthreads), *ptrs,
                          _ptr(sums, _dp))
    if not want_fields:
        return float(val)
    U, M, G, sg, ms = outs
    return float(val), dict(U=U, M=M, G=G, sigma=sg, measure=ms, sums=sums, virt=vg)


def nmi(U: np.ndarray, H: np.ndarray) -> float:
    """Normalised mutual information of two float images (or_nmi)."""
    lib = _load()
    u, h = _f32(U).ravel(), _f32(H).ravel()
    return float(lib.or_nmi(_ptr(u, _fp), _ptr(h, _fp), ctypes.c_longlong(u.size)))


def nmi_eval(fixed_geom: Geom, fixed: np.ndarray, moving_geom: Geom, moving: np.ndarray,
             virt_spacing: Sequence[float], mat, hr_moving: bool = True) -> float:
    """NMI of a 3D evaluation (PatchSize 0): fixed resampled through the
    identity and moving through ``mat`` onto the virtual grid, rounded to
    float32 as the device holds them; the ultrasound is the fixed image when
    hr_moving."""
    vg = virtual_geom(3, fixed_geom, virt_spacing)
    eye = np.eye(4, dtype=np.float32)
    F = resample(3, vg, fixed_geom, fixed, eye).astype(np.float32)
    M = resample(3, vg, moving_geom, moving, mat).astype(np.float32)
    return nmi(F, M) if hr_moving else nmi(M, F)


def affine3d(rot, trans, scale, shear, center, shift) -> np.ndarray:
    lib = _load()
    out = np.zeros(16, dtype=np.float32)
    args = [_f64(v) for v in (rot, trans, scale, shear, center, shift)]
    lib.or_affine3d(*[_ptr(a, _dp) for a in args], _ptr(out, _fp))
    return out.reshape(4, 4)


def affine2d(rot: float, trans, scale, shear: float, center, shift) -> np.ndarray:
    lib = _load()
    out = np.zeros(9, dtype=np.float32)
    t, s, c, sh = (_f64(v) for v in (trans, scale, center, shift))
    lib.or_affine2d(float(rot), _ptr(t, _dp), _ptr(s, _dp), float(shear), _ptr(c, _dp),
                    _ptr(sh, _dp), _ptr(out, _fp))
    return out.reshape(3, 3)
