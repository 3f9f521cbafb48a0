"""ctypes binding of liblc2.so (the C ABI in include/lc2.h).

Loading fails loudly when the library has not been built: there is no CPU
fallback for the LC2 path.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

from . import build as _build
from .geometry import Geometry

LC2_OK = 0
STATUS_NAMES = {
    0: "LC2_OK",
    1: "LC2_ERR_INVALID_ARGUMENT",
    2: "LC2_ERR_OUT_OF_MEMORY",
    3: "LC2_ERR_CUDA",
    4: "LC2_ERR_NOT_READY",
    5: "LC2_ERR_SINGULAR",
    6: "LC2_ERR_UNSUPPORTED",
    7: "LC2_ERR_TIMEOUT",
}
MODES = {"2D": 0, "3D": 1, "2DTo3D": 2}
OPTION_TILE_ROWS = 1
OPTION_ZCHUNK = 2
OPTION_GRAPHS = 3
OPTION_PIPELINE = 4
OPTION_STREAM_PRIORITY = 5
OPTION_STACK_BATCHING = 6
OPTION_GENERIC = 7
OPTION_PRESAMPLE = 8
STORAGE = {"f32": 0, "f16": 1, "bf16": 2}

# Every symbol include/lc2.h declares (checked by the test suite).
EXPORTED = [
    "lc2_create", "lc2_destroy", "lc2_set_images", "lc2_virtual_dims", "lc2_evaluate",
    "lc2_evaluate_batch", "lc2_stage_transforms", "lc2_launch_staged", "lc2_fetch_results",
    "lc2_get_stream", "lc2_set_stream", "lc2_evaluate_fields", "lc2_launch_count",
    "lc2_enable_kernel_timing", "lc2_kernel_times", "lc2_set_option", "lc2_wait_probe",
    "lc2_affine_3d", "lc2_affine_2d", "lc2_invert_affine_3d", "lc2_last_error", "lc2_version",
    "lc2_evaluate_noalloc", "lc2_minimize", "lc2_register", "lc2_params_to_matrix",
    "lc2_stack_create", "lc2_stack_destroy", "lc2_stack_set_moving", "lc2_stack_add_frame",
    "lc2_stack_frames", "lc2_stack_frame_context", "lc2_stack_evaluate", "lc2_stack_set_graphs",
    "lc2_stack_launch_count", "lc2_stack_graph_launches", "lc2_context_bytes",
    "lc2_server_create", "lc2_server_submit", "lc2_server_poll", "lc2_server_drain",
    "lc2_server_get_stats", "lc2_server_reset_stats", "lc2_server_destroy",
    "lc2_graph_launches", "lc2_autotune", "lc2_get_config", "lc2_weighting_map",
    "lc2_warp_affine_2d", "lc2_stack_register", "lc2_server_submit_stack",
    "lc2_server_poll_stack", "lc2_stack_set_option", "lc2_stack_get_option",
    "lc2_set_images_device", "lc2_merger_create", "lc2_merger_destroy", "lc2_merger_evaluate",
    "lc2_merger_launch_count", "lc2_debug_fail_allocation", "lc2_debug_device_bytes",
]

ALGORITHMS = {"direct_l": 1, "bobyqa": 2, "nelder_mead": 3, "quad_tr": 4}
ENTRIES = {"translation": 1, "rotation": 2, "scale": 4, "shear": 8}

OBSERVER = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double))
BATCH_OBJECTIVE = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_double),
                                   ctypes.POINTER(ctypes.c_double))


class lc2_opt_problem(ctypes.Structure):
    _fields_ = [("algorithm", ctypes.c_int), ("dim", ctypes.c_int),
                ("lower", ctypes.POINTER(ctypes.c_double)),
                ("upper", ctypes.POINTER(ctypes.c_double)), ("xtol_rel", ctypes.c_double),
                ("maxeval", ctypes.c_int), ("initial_step", ctypes.c_double)]


class lc2_opt_report(ctypes.Structure):
    _fields_ = [("evaluations", ctypes.c_int), ("batches", ctypes.c_int)]


class lc2_registration(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("initial", ctypes.c_double * 12),
                ("lower", ctypes.c_double * 12), ("upper", ctypes.c_double * 12),
                ("center", ctypes.c_float * 3), ("shift", ctypes.c_float * 3),
                ("direct_entries", ctypes.c_int), ("direct_maxeval", ctypes.c_int),
                ("rounds", ctypes.c_int), ("round_entries", ctypes.c_int * 8),
                ("round_xtol", ctypes.c_double * 8), ("round_maxeval", ctypes.c_int),
                ("local_algorithm", ctypes.c_int), ("lc2_of_matrices", BATCH_OBJECTIVE),
                ("user", ctypes.c_void_p), ("observer", ctypes.c_void_p),
                ("observer_user", ctypes.c_void_p), ("maximize", ctypes.c_int)]


class lc2_registration_result(ctypes.Structure):
    _fields_ = [("params", ctypes.c_double * 12), ("lc2", ctypes.c_double),
                ("evaluations", ctypes.c_int), ("launches", ctypes.c_int)]


class LC2Error(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class lc2_geometry(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int * 3), ("spacing", ctypes.c_float * 3),
                ("origin", ctypes.c_float * 3)]


class lc2_config(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("fixed", lc2_geometry), ("moving", lc2_geometry),
                ("virtual_spacing", ctypes.c_float * 3), ("patch_size", ctypes.c_int),
                ("high_res_is_moving", ctypes.c_int), ("storage", ctypes.c_int),
                ("max_batch", ctypes.c_int), ("device", ctypes.c_int)]


class lc2_server_config(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_size_t), ("max_active", ctypes.c_int),
                ("device", ctypes.c_int), ("merge_window_us", ctypes.c_int)]


class lc2_request(ctypes.Structure):
    _fields_ = [("config", lc2_config), ("fixed", ctypes.POINTER(ctypes.c_float)),
                ("moving", ctypes.POINTER(ctypes.c_float)), ("registration", lc2_registration)]


class lc2_request_result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("message", ctypes.c_char * 160),
                ("result", lc2_registration_result), ("queue_ms", ctypes.c_double),
                ("run_ms", ctypes.c_double), ("total_ms", ctypes.c_double),
                ("device_bytes", ctypes.c_size_t), ("admission", ctypes.c_longlong)]


class lc2_stack_request(ctypes.Structure):
    _fields_ = [("moving", lc2_geometry), ("moving_image", ctypes.POINTER(ctypes.c_float)),
                ("patch_size", ctypes.c_int), ("storage", ctypes.c_int), ("frames", ctypes.c_int),
                ("frame_geoms", ctypes.POINTER(lc2_geometry)),
                ("frame_images", ctypes.POINTER(ctypes.POINTER(ctypes.c_float))),
                ("virtual_spacing", ctypes.c_float * 3),
                ("registrations", ctypes.POINTER(lc2_registration))]


class lc2_server_stats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_longlong), ("completed", ctypes.c_longlong),
                ("failed", ctypes.c_longlong), ("queued", ctypes.c_int), ("active", ctypes.c_int),
                ("peak_active", ctypes.c_int), ("budget_bytes", ctypes.c_size_t),
                ("bytes_in_use", ctypes.c_size_t), ("peak_bytes", ctypes.c_size_t),
                ("p50_ms", ctypes.c_double), ("p95_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double),
                ("elapsed_s", ctypes.c_double), ("merged_launches", ctypes.c_longlong),
                ("merged_steps", ctypes.c_longlong)]


_fp = ctypes.POINTER(ctypes.c_float)
_dp = ctypes.POINTER(ctypes.c_double)
_lib = None


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load liblc2.so (building it with nvcc if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if build_if_missing and _build.needs_build():
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"liblc2.so is not built ({path}); run lc2registration_gb300.build")
    lib = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    sig = {
        "lc2_create": ([ctypes.POINTER(lc2_config), ctypes.POINTER(vp)], ctypes.c_int),
        "lc2_destroy": ([vp], ctypes.c_int),
        "lc2_set_images": ([vp, _fp, _fp], ctypes.c_int),
        "lc2_set_images_device": ([vp, vp, vp], ctypes.c_int),
        "lc2_merger_create": ([ctypes.c_int, ctypes.POINTER(vp)], ctypes.c_int),
        "lc2_merger_destroy": ([vp], ctypes.c_int),
        "lc2_merger_evaluate": ([vp, ctypes.c_int, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_int),
                                 _fp, _dp], ctypes.c_int),
        "lc2_merger_launch_count": ([vp], ctypes.c_longlong),
        "lc2_debug_fail_allocation": ([ctypes.c_longlong], ctypes.c_int),
        "lc2_debug_device_bytes": ([ctypes.POINTER(ctypes.c_size_t),
                                    ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
        "lc2_virtual_dims": ([vp, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "lc2_evaluate": ([vp, _fp, _dp], ctypes.c_int),
        "lc2_evaluate_batch": ([vp, _fp, ctypes.c_int, _dp], ctypes.c_int),
        "lc2_stage_transforms": ([vp, _fp, ctypes.c_int], ctypes.c_int),
        "lc2_launch_staged": ([vp, ctypes.c_int], ctypes.c_int),
        "lc2_fetch_results": ([vp, _dp, ctypes.c_int], ctypes.c_int),
        "lc2_get_stream": ([vp], vp),
        "lc2_set_stream": ([vp, vp], ctypes.c_int),
        "lc2_evaluate_fields": ([vp, _fp, _dp, _fp, _fp, _fp, _fp, _fp], ctypes.c_int),
        "lc2_launch_count": ([vp], ctypes.c_longlong),
        "lc2_enable_kernel_timing": ([vp, ctypes.c_int], ctypes.c_int),
        "lc2_wait_probe": ([vp], ctypes.c_int),
        "lc2_set_option": ([vp, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "lc2_kernel_times": ([vp, _dp, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
        "lc2_affine_3d": ([_fp, _fp, _fp, _fp, _fp, _fp, _fp], ctypes.c_int),
        "lc2_affine_2d": ([ctypes.c_float, _fp, _fp, ctypes.c_float, _fp, _fp, _fp], ctypes.c_int),
        "lc2_invert_affine_3d": ([_fp, _fp], ctypes.c_int),
        "lc2_last_error": ([], ctypes.c_char_p),
        "lc2_version": ([], ctypes.c_char_p),
        "lc2_minimize": ([ctypes.POINTER(lc2_opt_problem), BATCH_OBJECTIVE, vp, _dp, _dp,
                          ctypes.POINTER(lc2_opt_report)], ctypes.c_int),
        "lc2_register": ([vp, ctypes.POINTER(lc2_registration),
                          ctypes.POINTER(lc2_registration_result)], ctypes.c_int),
        "lc2_params_to_matrix": ([ctypes.c_int, _dp, _fp, _fp, _fp], ctypes.c_int),
        "lc2_evaluate_noalloc": ([ctypes.c_int, ctypes.POINTER(lc2_geometry),
                                  ctypes.POINTER(lc2_geometry), ctypes.c_int, vp, vp, _fp, vp,
                                  vp], ctypes.c_int),
        "lc2_stack_create": ([ctypes.POINTER(lc2_geometry), ctypes.c_int, ctypes.c_int,
                              ctypes.c_int, ctypes.POINTER(vp)], ctypes.c_int),
        "lc2_stack_destroy": ([vp], ctypes.c_int),
        "lc2_stack_set_moving": ([vp, _fp], ctypes.c_int),
        "lc2_stack_add_frame": ([vp, ctypes.POINTER(lc2_geometry), _fp, _fp,
                                 ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "lc2_stack_frames": ([vp], ctypes.c_int),
        "lc2_stack_frame_context": ([vp, ctypes.c_int, ctypes.POINTER(vp)], ctypes.c_int),
        "lc2_stack_evaluate": ([vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _fp, _dp],
                               ctypes.c_int),
        "lc2_stack_set_graphs": ([vp, ctypes.c_int], ctypes.c_int),
        "lc2_stack_launch_count": ([vp], ctypes.c_longlong),
        "lc2_stack_graph_launches": ([vp], ctypes.c_longlong),
        "lc2_stack_register": ([vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                ctypes.POINTER(lc2_registration),
                                ctypes.POINTER(lc2_registration_result),
                                ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong)],
                               ctypes.c_int),
        "lc2_context_bytes": ([ctypes.POINTER(lc2_config), ctypes.POINTER(ctypes.c_size_t),
                               ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
        "lc2_server_create": ([ctypes.POINTER(lc2_server_config), ctypes.POINTER(vp)],
                              ctypes.c_int),
        "lc2_server_submit": ([vp, ctypes.POINTER(lc2_request), ctypes.POINTER(ctypes.c_longlong)],
                              ctypes.c_int),
        "lc2_server_poll": ([vp, ctypes.c_longlong, ctypes.c_int,
                             ctypes.POINTER(lc2_request_result)], ctypes.c_int),
        "lc2_server_drain": ([vp, ctypes.c_int], ctypes.c_int),
        "lc2_server_get_stats": ([vp, ctypes.POINTER(lc2_server_stats)], ctypes.c_int),
        "lc2_server_reset_stats": ([vp], ctypes.c_int),
        "lc2_server_destroy": ([vp], ctypes.c_int),
        "lc2_server_submit_stack": ([vp, ctypes.POINTER(lc2_stack_request),
                                     ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
        "lc2_server_poll_stack": ([vp, ctypes.c_longlong, ctypes.c_int,
                                   ctypes.POINTER(lc2_request_result), ctypes.c_int],
                                  ctypes.c_int),
        "lc2_stack_set_option": ([vp, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "lc2_stack_get_option": ([vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "lc2_graph_launches": ([vp], ctypes.c_longlong),
        "lc2_get_config": ([vp, ctypes.POINTER(lc2_config)], ctypes.c_int),
        "lc2_weighting_map": ([vp, _fp, _dp, _fp], ctypes.c_int),
        "lc2_warp_affine_2d": ([_fp, ctypes.c_int, ctypes.c_int, _fp, ctypes.c_int, ctypes.c_int,
                                _dp, ctypes.c_int], ctypes.c_int),
        "lc2_autotune": ([vp, _fp, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                          ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _check(status: int):
    if status != LC2_OK:
        raise LC2Error(status, load().lc2_last_error().decode())


def _geom(g: Geometry) -> lc2_geometry:
    out = lc2_geometry()
    for a in range(3):
        out.dim[a] = int(g.dim[a])
        out.spacing[a] = float(g.spacing[a])
        out.origin[a] = float(g.origin[a])
    return out


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def make_config(mode: str, fixed_geom: Geometry, moving_geom: Geometry,
                virt_spacing: Sequence[float], patch_size: int, high_res_is_moving: bool = True,
                storage: str = "f32", max_batch: int = 0, device: int = 0) -> lc2_config:
    cfg = lc2_config()
    cfg.mode = MODES[mode]
    cfg.fixed = _geom(fixed_geom)
    cfg.moving = _geom(moving_geom)
    vs = list(virt_spacing) + [1.0] * (3 - len(virt_spacing))
    for a in range(3):
        cfg.virtual_spacing[a] = float(vs[a])
    cfg.patch_size = int(patch_size)
    cfg.high_res_is_moving = int(bool(high_res_is_moving))
    cfg.storage = STORAGE[storage]
    cfg.max_batch = int(max_batch)
    cfg.device = int(device)
    return cfg


def context_bytes(cfg: lc2_config):
    """(held, peak) device bytes of a context of this configuration."""
    held, peak = ctypes.c_size_t(), ctypes.c_size_t()
    _check(load().lc2_context_bytes(ctypes.byref(cfg), ctypes.byref(held), ctypes.byref(peak)))
    return held.value, peak.value


class Context:
    """One LC2 evaluation context (fixed + moving image on one GPU)."""

    def __init__(self, mode: str, fixed_geom: Geometry, moving_geom: Geometry,
                 virt_spacing: Sequence[float], patch_size: int, high_res_is_moving: bool = True,
                 storage: str = "f32", max_batch: int = 0, device: int = 0):
        lib = load()
        cfg = make_config(mode, fixed_geom, moving_geom, virt_spacing, patch_size,
                          high_res_is_moving, storage, max_batch, device)
        self.mode = mode
        self.matrix_size = 9 if mode == "2D" else 16
        self._h = ctypes.c_void_p()
        _check(lib.lc2_create(ctypes.byref(cfg), ctypes.byref(self._h)))
        self._lib = lib

    def close(self):
        if self._h:
            self._lib.lc2_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_images(self, fixed: np.ndarray, moving: np.ndarray):
        f, m = _f32(fixed), _f32(moving)
        _check(self._lib.lc2_set_images(self._h, f.ctypes.data_as(_fp), m.ctypes.data_as(_fp)))

    def set_images_device(self, fixed_ptr: int, moving_ptr: int):
        """lc2_set_images from device pointers (float32 on the context's device)."""
        _check(self._lib.lc2_set_images_device(self._h, ctypes.c_void_p(fixed_ptr),
                                               ctypes.c_void_p(moving_ptr)))

    def virtual_dims(self):
        d = (ctypes.c_int * 3)()
        _check(self._lib.lc2_virtual_dims(self._h, d))
        return tuple(d)

    def _mats(self, mats) -> np.ndarray:
        m = _f32(mats).reshape(-1, self.matrix_size)
        return m

    def evaluate(self, mat) -> float:
        m = self._mats(mat)
        out = ctypes.c_double()
        _check(self._lib.lc2_evaluate(self._h, m.ctypes.data_as(_fp), ctypes.byref(out)))
        return out.value

    def evaluate_batch(self, mats) -> np.ndarray:
        m = self._mats(mats)
        out = np.empty(m.shape[0], dtype=np.float64)
        _check(self._lib.lc2_evaluate_batch(self._h, m.ctypes.data_as(_fp), m.shape[0],
                                            out.ctypes.data_as(_dp)))
        return out

    def stage(self, mats) -> int:
        m = self._mats(mats)
        _check(self._lib.lc2_stage_transforms(self._h, m.ctypes.data_as(_fp), m.shape[0]))
        return m.shape[0]

    def launch(self, count: int):
        _check(self._lib.lc2_launch_staged(self._h, int(count)))

    def fetch(self, count: int) -> np.ndarray:
        out = np.empty(count, dtype=np.float64)
        _check(self._lib.lc2_fetch_results(self._h, out.ctypes.data_as(_dp), int(count)))
        return out

    def stream(self) -> int:
        return self._lib.lc2_get_stream(self._h) or 0

    def set_stream(self, stream_ptr: Optional[int]):
        _check(self._lib.lc2_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    def launch_count(self) -> int:
        return int(self._lib.lc2_launch_count(self._h))

    def set_option(self, option: int, value: int):
        _check(self._lib.lc2_set_option(self._h, int(option), int(value)))

    def weighting_map(self, mat):
        """(lc2, per-voxel measure / sigma float32 array)."""
        m = self._mats(mat)
        d = self.virtual_dims()
        out = np.empty(d[0] * d[1] * d[2], dtype=np.float32)
        v = ctypes.c_double()
        _check(self._lib.lc2_weighting_map(self._h, m.ctypes.data_as(_fp), ctypes.byref(v),
                                           out.ctypes.data_as(_fp)))
        return v.value, out

    def graph_launches(self) -> int:
        return int(self._lib.lc2_graph_launches(self._h))

    def autotune(self, mats):
        """Times the fused kernel's tilings on these transforms, keeps the
        fastest; returns (tile_rows, zchunk)."""
        m = self._mats(mats)
        tr, zc = ctypes.c_int(), ctypes.c_int()
        _check(self._lib.lc2_autotune(self._h, m.ctypes.data_as(_fp), m.shape[0],
                                      ctypes.byref(tr), ctypes.byref(zc)))
        return tr.value, zc.value

    def wait_probe(self):
        """Self-test of the bounded device-side waits (lc2_wait_probe): raises
        LC2Error(LC2_ERR_TIMEOUT) when the one-second wait expired and was
        reported, as it must; the context stays usable."""
        _check(self._lib.lc2_wait_probe(self._h))

    def enable_kernel_timing(self, on: bool = True):
        _check(self._lib.lc2_enable_kernel_timing(self._h, int(bool(on))))

    def kernel_times(self):
        """{'warp'|'sobel'|'moments': (total ms, launches)} since the last call."""
        ms = (ctypes.c_double * 3)()
        cnt = (ctypes.c_longlong * 3)()
        _check(self._lib.lc2_kernel_times(self._h, ms, cnt))
        return {k: (ms[i], int(cnt[i])) for i, k in enumerate(("warp", "sobel", "moments"))}

    def evaluate_fields(self, mat):
        """Returns (lc2, dict of per-voxel float32 fields U, M, G, sigma, measure)."""
        m = self._mats(mat)
        d = self.virtual_dims()
        n = d[0] * d[1] * d[2]
        f = {k: np.empty(n, dtype=np.float32) for k in ("U", "M", "G", "sigma", "measure")}
        out = ctypes.c_double()
        _check(self._lib.lc2_evaluate_fields(
            self._h, m.ctypes.data_as(_fp), ctypes.byref(out),
            *[f[k].ctypes.data_as(_fp) for k in ("U", "M", "G", "sigma", "measure")]))
        return out.value, f


class FrameView(Context):
    """A stack frame's own context (owned by the stack: never destroyed here)."""

    def __init__(self, lib, handle):
        self._lib = lib
        self._h = handle
        self.mode = "2DTo3D"
        self.matrix_size = 16

    def close(self):
        self._h = ctypes.c_void_p()


class Merger:
    """lc2_merger_*: evaluations of several contexts in one launch."""

    def __init__(self, device: int = 0):
        self._lib = load()
        h = ctypes.c_void_p()
        _check(self._lib.lc2_merger_create(int(device), ctypes.byref(h)))
        self._h = h

    def evaluate(self, contexts, mats_per_context):
        """contexts: list of Context; mats_per_context: list of (count, 3|4, 3|4)
        arrays. Returns a list of LC2 arrays, one per context."""
        n = len(contexts)
        counts = [len(m) for m in mats_per_context]
        flat = np.ascontiguousarray(np.concatenate(
            [np.asarray(m, dtype=np.float32).reshape(len(m), -1) for m in mats_per_context]),
            dtype=np.float32)
        out = np.empty(sum(counts), dtype=np.float64)
        hs = (ctypes.c_void_p * n)(*[c.handle.value for c in contexts])
        cs = (ctypes.c_int * n)(*counts)
        _check(self._lib.lc2_merger_evaluate(self._h, n, hs, cs, flat.ctypes.data_as(_fp),
                                             out.ctypes.data_as(_dp)))
        res, k = [], 0
        for c in counts:
            res.append(out[k:k + c])
            k += c
        return res

    def launch_count(self) -> int:
        return int(self._lib.lc2_merger_launch_count(self._h))

    def close(self):
        if self._h:
            self._lib.lc2_merger_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Stack:
    """A 2D-to-3D frame stack: one moving volume, ultrasound frames of their
    own sizes, evaluations of (frame, pose) pairs in one launch."""

    def __init__(self, moving_geom: Geometry, patch_size: int, storage: str = "f32",
                 device: int = 0):
        lib = load()
        self._lib = lib
        self._h = ctypes.c_void_p()
        g = _geom(moving_geom)
        _check(lib.lc2_stack_create(ctypes.byref(g), int(patch_size), STORAGE[storage],
                                    int(device), ctypes.byref(self._h)))

    def close(self):
        if self._h:
            self._lib.lc2_stack_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_moving(self, moving: np.ndarray):
        m = _f32(moving)
        _check(self._lib.lc2_stack_set_moving(self._h, m.ctypes.data_as(_fp)))

    def add_frame(self, frame_geom: Geometry, virt_spacing, ultrasound: np.ndarray) -> int:
        g = _geom(frame_geom)
        vs = _f32(list(virt_spacing) + [1.0] * (3 - len(virt_spacing)))
        u = _f32(ultrasound)
        fid = ctypes.c_int()
        _check(self._lib.lc2_stack_add_frame(self._h, ctypes.byref(g), vs.ctypes.data_as(_fp),
                                             u.ctypes.data_as(_fp), ctypes.byref(fid)))
        return fid.value

    def frames(self) -> int:
        return int(self._lib.lc2_stack_frames(self._h))

    def frame_context(self, frame_id: int) -> "FrameView":
        h = ctypes.c_void_p()
        _check(self._lib.lc2_stack_frame_context(self._h, int(frame_id), ctypes.byref(h)))
        return FrameView(self._lib, h)

    def evaluate(self, frame_ids, mats) -> np.ndarray:
        ids = np.ascontiguousarray(frame_ids, dtype=np.int32)
        m = _f32(mats).reshape(-1, 16)
        if m.shape[0] != ids.shape[0]:
            raise ValueError("one matrix per frame id")
        out = np.empty(ids.shape[0], dtype=np.float64)
        _check(self._lib.lc2_stack_evaluate(self._h, ids.shape[0],
                                            ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                            m.ctypes.data_as(_fp), out.ctypes.data_as(_dp)))
        return out

    def set_graphs(self, on: bool):
        _check(self._lib.lc2_stack_set_graphs(self._h, int(bool(on))))

    def set_option(self, option: int, value: int):
        _check(self._lib.lc2_stack_set_option(self._h, int(option), int(value)))

    def register(self, frame_ids, registrations):
        """lc2_stack_register: registrations = list of make_registration
        keyword dicts (mode is 2DTo3D), one per frame id. Returns (list of
        result dicts, stack launches)."""
        n = len(frame_ids)
        ids = (ctypes.c_int * n)(*[int(i) for i in frame_ids])
        regs = (lc2_registration * n)()
        keep = []
        for i, kw in enumerate(registrations):
            regs[i] = make_registration("2DTo3D", keep=keep, **kw)
        res = (lc2_registration_result * n)()
        sts = (ctypes.c_int * n)()
        launches = ctypes.c_longlong()
        _check(self._lib.lc2_stack_register(self._h, n, ids, regs, res, sts,
                                            ctypes.byref(launches)))
        out = [dict(params=np.array(r.params[:12]), lc2=r.lc2, evaluations=r.evaluations,
                    launches=r.launches) for r in res]
        return out, launches.value

    def launch_count(self) -> int:
        return int(self._lib.lc2_stack_launch_count(self._h))

    def weighting_map(self, mat):
        """(lc2, per-voxel measure / sigma float32 array)."""
        m = self._mats(mat)
        d = self.virtual_dims()
        out = np.empty(d[0] * d[1] * d[2], dtype=np.float32)
        v = ctypes.c_double()
        _check(self._lib.lc2_weighting_map(self._h, m.ctypes.data_as(_fp), ctypes.byref(v),
                                           out.ctypes.data_as(_fp)))
        return v.value, out

    def graph_launches(self) -> int:
        return int(self._lib.lc2_stack_graph_launches(self._h))


def affine_3d(rot, trans, scale=(1, 1, 1), shear=(0, 0, 0), center=(0, 0, 0), shift=(0, 0, 0)):
    lib = load()
    args = [_f32(v) for v in (rot, trans, scale, shear, center, shift)]
    out = np.zeros(16, dtype=np.float32)
    _check(lib.lc2_affine_3d(*[a.ctypes.data_as(_fp) for a in args], out.ctypes.data_as(_fp)))
    return out.reshape(4, 4)


def affine_2d(rot, trans, scale=(1, 1), shear=0.0, center=(0, 0), shift=(0, 0)):
    lib = load()
    t, s, c, sh = (_f32(v) for v in (trans, scale, center, shift))
    out = np.zeros(9, dtype=np.float32)
    _check(lib.lc2_affine_2d(float(rot), t.ctypes.data_as(_fp), s.ctypes.data_as(_fp), float(shear),
                             c.ctypes.data_as(_fp), sh.ctypes.data_as(_fp), out.ctypes.data_as(_fp)))
    return out.reshape(3, 3)


def warp_affine_2d(src: np.ndarray, dst_shape, coeffs, device: int = 0) -> np.ndarray:
    """lc2_warp_affine_2d: src (h, w) float image warped by the forward pixel
    map coeffs (2x3) into an array of dst_shape (h', w')."""
    lib = load()
    s = _f32(src)
    sh, sw = s.shape
    dh, dw = dst_shape
    out = np.empty((dh, dw), dtype=np.float32)
    c = np.ascontiguousarray(coeffs, dtype=np.float64).ravel()
    _check(lib.lc2_warp_affine_2d(s.ctypes.data_as(_fp), sw, sh, out.ctypes.data_as(_fp), dw, dh,
                                  c.ctypes.data_as(_dp), int(device)))
    return out


def invert_affine_3d(mat) -> np.ndarray:
    lib = load()
    m = _f32(mat).ravel()
    out = np.zeros(16, dtype=np.float32)
    _check(lib.lc2_invert_affine_3d(m.ctypes.data_as(_fp), out.ctypes.data_as(_fp)))
    return out.reshape(4, 4)


def minimize(fun_batch, x0, lower, upper, algorithm: str = "bobyqa", xtol_rel: float = 1e-4,
             maxeval: int = 0, initial_step: float = 0.0):
    """Runs lc2_minimize with a Python batch objective fun_batch(X[count, dim]) -> f[count].
    Returns (x, fmin, evaluations, batches)."""
    lib = load()
    n = len(x0)
    lo = np.ascontiguousarray(lower, dtype=np.float64)
    hi = np.ascontiguousarray(upper, dtype=np.float64)
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    err = []

    def cb(user, count, dim, xp, fp):
        try:
            X = np.ctypeslib.as_array(xp, shape=(count * dim,)).reshape(count, dim).copy()
            F = np.asarray(fun_batch(X), dtype=np.float64)
            np.ctypeslib.as_array(fp, shape=(count,))[:] = F
            return 0
        except Exception as e:  # surfaced after the call
            err.append(e)
            return 1

    cfun = BATCH_OBJECTIVE(cb)
    p = lc2_opt_problem(ALGORITHMS[algorithm], n, lo.ctypes.data_as(_dp), hi.ctypes.data_as(_dp),
                        float(xtol_rel), int(maxeval), float(initial_step))
    rep = lc2_opt_report()
    fmin = ctypes.c_double()
    st = lib.lc2_minimize(ctypes.byref(p), cfun, None, x.ctypes.data_as(_dp), ctypes.byref(fmin),
                          ctypes.byref(rep))
    if err:
        raise err[0]
    _check(st)
    return x, fmin.value, rep.evaluations, rep.batches


def _mask(entries) -> int:
    if isinstance(entries, int):
        return entries
    m = 0
    for e in entries:
        m |= ENTRIES[e]
    return m


def register(ctx, initial, lower, upper, center, shift=(0.0, 0.0, 0.0), direct_entries=(),
             direct_maxeval: int = 50, rounds=(), round_maxeval: int = 0,
             local_algorithm: str = "bobyqa", mode: Optional[str] = None, lc2_of_matrices=None,
             observer=None, maximize: bool = False):
    """lc2_register: DIRECT on direct_entries, then local rounds [(entries, xtol), ...].

    ctx: a Context (GPU objective) or None together with lc2_of_matrices, a
    Python function mapping a (count, 9|16) float64 array of matrices to LC2
    values (e.g. the FP64 oracle), and mode. observer(stage, params (count, n),
    lc2 (count,)) sees every evaluation. Returns dict(params, lc2,
    evaluations, launches)."""
    lib = load()
    mode = mode or ctx.mode
    err = []
    keep = []
    reg = make_registration(mode, initial, lower, upper, center, shift, direct_entries,
                            direct_maxeval, rounds, round_maxeval, local_algorithm,
                            lc2_of_matrices, observer, err, keep, maximize)
    out = lc2_registration_result()
    st = lib.lc2_register(ctx.handle if ctx is not None else None, ctypes.byref(reg),
                          ctypes.byref(out))
    if err:
        raise err[0]
    _check(st)
    n = 6 if mode == "2D" else 12
    return dict(params=np.array(out.params[:n]), lc2=out.lc2, evaluations=out.evaluations,
                launches=out.launches)


def make_registration(mode, initial, lower, upper, center, shift=(0.0, 0.0, 0.0),
                      direct_entries=(), direct_maxeval: int = 50, rounds=(),
                      round_maxeval: int = 0, local_algorithm: str = "bobyqa",
                      lc2_of_matrices=None, observer=None, err=None, keep=None,
                      maximize: bool = False):
    """An lc2_registration struct. Python callbacks append their exceptions to
    err; the ctypes callback objects are appended to keep, which the caller
    holds while the struct is in use."""
    err = [] if err is None else err
    keep = [] if keep is None else keep
    reg = lc2_registration()
    reg.mode = MODES[mode]
    n = 6 if mode == "2D" else 12
    for i in range(n):
        reg.initial[i] = float(initial[i])
        reg.lower[i] = float(lower[i])
        reg.upper[i] = float(upper[i])
    for a in range(min(3, len(center))):
        reg.center[a] = float(center[a])
    for a in range(min(3, len(shift))):
        reg.shift[a] = float(shift[a])
    reg.direct_entries = _mask(direct_entries)
    reg.direct_maxeval = int(direct_maxeval)
    reg.rounds = len(rounds)
    for r, (entries, xtol) in enumerate(rounds):
        reg.round_entries[r] = _mask(entries)
        reg.round_xtol[r] = float(xtol)
    reg.round_maxeval = int(round_maxeval)
    reg.local_algorithm = ALGORITHMS[local_algorithm]
    reg.maximize = int(bool(maximize))
    if lc2_of_matrices is not None:
        def cb(user, count, dim, xp, fp):
            try:
                M = np.ctypeslib.as_array(xp, shape=(count * dim,)).reshape(count, dim).copy()
                np.ctypeslib.as_array(fp, shape=(count,))[:] = lc2_of_matrices(M)
                return 0
            except Exception as e:
                err.append(e)
                return 1
        fn = BATCH_OBJECTIVE(cb)
        keep.append(fn)  # the struct holds only the function pointer
        reg.lc2_of_matrices = fn
    if observer is not None:
        def ob(user, stage, count, nparams, pp, lp):
            try:
                P = np.ctypeslib.as_array(pp, shape=(count * nparams,)).reshape(count, nparams)
                observer(stage, P.copy(), np.ctypeslib.as_array(lp, shape=(count,)).copy())
            except Exception as e:  # an observer cannot fail the C driver
                err.append(e)
        ob_c = OBSERVER(ob)
        keep.append(ob_c)
        reg.observer = ctypes.cast(ob_c, ctypes.c_void_p)
    return reg


def params_to_matrix(mode: str, params, center, shift=(0.0, 0.0, 0.0)) -> np.ndarray:
    lib = load()
    n = 6 if mode == "2D" else 12
    p = np.zeros(12, dtype=np.float64)
    p[:n] = params[:n]
    c = np.zeros(3, dtype=np.float32)
    c[:len(center)] = center[:3]
    sh = np.zeros(3, dtype=np.float32)
    sh[:len(shift)] = shift[:3]
    m = np.zeros(9 if mode == "2D" else 16, dtype=np.float32)
    _check(lib.lc2_params_to_matrix(MODES[mode], p.ctypes.data_as(_dp), c.ctypes.data_as(_fp),
                                    sh.ctypes.data_as(_fp), m.ctypes.data_as(_fp)))
    return m.reshape(3, 3) if mode == "2D" else m.reshape(4, 4)


class Server:
    """lc2_server_*: registrations admitted by device-memory budget, run
    concurrently on worker threads, results polled by ticket."""

    def __init__(self, budget_bytes: int = 0, max_active: int = 0, device: int = 0,
                 merge_window_us: int = 0):
        lib = load()
        self._lib = lib
        self._h = ctypes.c_void_p()
        cfg = lc2_server_config(int(budget_bytes), int(max_active), int(device),
                                int(merge_window_us))
        _check(lib.lc2_server_create(ctypes.byref(cfg), ctypes.byref(self._h)))
        self._keep = {}   # ticket -> callback objects the C side may still call
        self._errs = {}
        self._stack_n = {}  # ticket -> frames of a stack request

    def close(self):
        if self._h:
            self._lib.lc2_server_destroy(self._h)
            self._h = ctypes.c_void_p()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, cfg: lc2_config, fixed=None, moving=None, **registration) -> int:
        """Queues one registration; registration holds make_registration's
        arguments (initial, lower, upper, center, ...; mode is taken from cfg)."""
        mode = {v: k for k, v in MODES.items()}[cfg.mode]
        err, keep = [], []
        reg = make_registration(mode, err=err, keep=keep, **registration)
        req = lc2_request()
        req.config = cfg
        imgs = []
        if fixed is not None:
            f, m = _f32(fixed), _f32(moving)
            imgs = [f, m]
            req.fixed = f.ctypes.data_as(_fp)
            req.moving = m.ctypes.data_as(_fp)
        req.registration = reg
        t = ctypes.c_longlong()
        _check(self._lib.lc2_server_submit(self._h, ctypes.byref(req), ctypes.byref(t)))
        del imgs  # copied by the server
        self._keep[t.value] = keep
        self._errs[t.value] = err
        return t.value

    def poll(self, ticket: int, wait_ms: int = -1):
        """The result dict, or None while the request is queued or running."""
        out = lc2_request_result()
        st = self._lib.lc2_server_poll(self._h, int(ticket), int(wait_ms), ctypes.byref(out))
        if st == 4:
            return None
        _check(st)
        self._keep.pop(ticket, None)
        err = self._errs.pop(ticket, [])
        if err:
            raise err[0]
        r = out.result
        return dict(status=out.status, message=out.message.decode(), params=np.array(r.params[:]),
                    lc2=r.lc2, evaluations=r.evaluations, launches=r.launches,
                    queue_ms=out.queue_ms, run_ms=out.run_ms, total_ms=out.total_ms,
                    device_bytes=out.device_bytes, admission=out.admission)

    def submit_stack(self, moving_geom: Geometry, moving, patch_size: int, frames,
                     virt_spacing, registrations, storage: str = "f32") -> int:
        """One 2D-to-3D stack request: frames = [(Geometry, image)], one
        make_registration keyword dict per frame."""
        n = len(frames)
        req = lc2_stack_request()
        req.moving = _geom(moving_geom)
        mv = _f32(moving)
        req.moving_image = mv.ctypes.data_as(_fp)
        req.patch_size = int(patch_size)
        req.storage = STORAGE[storage]
        req.frames = n
        geoms = (lc2_geometry * n)(*[_geom(g) for g, _ in frames])
        imgs = [_f32(im) for _, im in frames]
        ptrs = (ctypes.POINTER(ctypes.c_float) * n)(*[im.ctypes.data_as(_fp) for im in imgs])
        req.frame_geoms = geoms
        req.frame_images = ptrs
        vs = list(virt_spacing) + [1.0] * (3 - len(virt_spacing))
        for a in range(3):
            req.virtual_spacing[a] = float(vs[a])
        regs = (lc2_registration * n)()
        keep = []
        for i, kw in enumerate(registrations):
            regs[i] = make_registration("2DTo3D", keep=keep, **kw)
        req.registrations = regs
        t = ctypes.c_longlong()
        _check(self._lib.lc2_server_submit_stack(self._h, ctypes.byref(req), ctypes.byref(t)))
        self._keep[t.value] = keep
        self._stack_n[t.value] = n
        return t.value

    def poll_stack(self, ticket: int, wait_ms: int = -1):
        """Per-frame result dicts, or None while the request is queued or running."""
        n = self._stack_n.get(ticket, 1)
        out = (lc2_request_result * n)()
        st = self._lib.lc2_server_poll_stack(self._h, int(ticket), int(wait_ms), out, n)
        if st == 4:
            return None
        _check(st)
        self._keep.pop(ticket, None)
        return [dict(status=o.status, message=o.message.decode(), params=np.array(o.result.params[:]),
                     lc2=o.result.lc2, evaluations=o.result.evaluations, queue_ms=o.queue_ms,
                     run_ms=o.run_ms, total_ms=o.total_ms, admission=o.admission) for o in out]

    def drain(self, wait_ms: int = -1) -> bool:
        st = self._lib.lc2_server_drain(self._h, int(wait_ms))
        if st == 4:
            return False
        _check(st)
        return True

    def stats(self) -> dict:
        st = lc2_server_stats()
        _check(self._lib.lc2_server_get_stats(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in lc2_server_stats._fields_}

    def reset_stats(self):
        _check(self._lib.lc2_server_reset_stats(self._h))
