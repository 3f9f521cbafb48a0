"""lc2_evaluate_noalloc: LC2 for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc: a host application whose own allocator
or memory pool owns the device heap, a real-time loop that must not allocate
after start-up, a plug-in that is handed device buffers and nothing else. For
them the library offers an entry point whose working memory is a fixed-size
static device array. This test hands it device buffers (allocated here, by
the test) and checks, through the C ABI, that its LC2 values agree with the
context entry point lc2_evaluate and with the FP64 oracle on consecutive
calls, in each of the three modes.
"""
import ctypes

import numpy as np
import pytest

from lc2registration_gb300 import capi, synth
from tests.helpers import oracle_eval, perturbed

pytestmark = pytest.mark.gpu

REL = 1e-5  # the LC2 tolerance used throughout the GPU tests


def _geom(dim, spacing, origin):
    g = capi.lc2_geometry()
    for a in range(3):
        g.dim[a] = int(dim[a])
        g.spacing[a] = float(spacing[a])
        g.origin[a] = float(origin[a])
    return g


def _noalloc(lib, mode, case, d_us, d_mov, mat, d_out, stream):
    vg = _geom(case.fixed_geom.dim, case.fixed_geom.spacing, case.fixed_geom.origin)
    mg = _geom(case.moving_geom.dim, case.moving_geom.spacing, case.moving_geom.origin)
    m = np.ascontiguousarray(mat, dtype=np.float32).ravel()
    return lib.lc2_evaluate_noalloc(capi.MODES[mode], ctypes.byref(vg), ctypes.byref(mg), case.r,
                                    ctypes.c_void_p(d_us.data_ptr()),
                                    ctypes.c_void_p(d_mov.data_ptr()),
                                    m.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                    ctypes.c_void_p(d_out.data_ptr()), ctypes.c_void_p(stream))


def _case(mode):
    if mode == "2D":
        return synth.case_2d(seed=61, size=64, r=3)
    if mode == "3D":
        return synth.case_3d(seed=62, mr_size=40, us_size=32, r=2, blobs=5)
    # 2D-to-3D: one ultrasound frame sliced from a 3D volume; the frame's own
    # spacing is the virtual spacing, so the frame is already on the virtual grid
    mr_case = synth.case_3d(seed=63, mr_size=40, us_size=32, r=3, blobs=5)
    return synth.frame_stack(mr_case.moving, mr_case.moving_geom, 1, seed=64, sides=(48,),
                             spacing=0.5, r=3)[0]


@pytest.mark.parametrize("mode", ["2D", "3D", "2DTo3D"])
def test_noalloc_matches_context_entry_point(mode):
    import torch

    lib = capi.load()
    case = _case(mode)
    # the virtual grid is the fixed grid (same spacing and origin), so the
    # ultrasound on the virtual grid is the fixed image itself
    ctx = capi.Context(case.mode, case.fixed_geom, case.moving_geom, case.virt_spacing, case.r)
    ctx.set_images(case.fixed, case.moving)
    mats = [case.true_mat] + list(perturbed(case, np.random.default_rng(3), 1))
    ref = [ctx.evaluate(m) for m in mats]
    orc = [oracle_eval(case, m) for m in mats]

    dev = torch.device("cuda:0")
    d_us = torch.from_numpy(np.ascontiguousarray(case.fixed, np.float32)).to(dev)
    d_mov = torch.from_numpy(np.ascontiguousarray(case.moving, np.float32)).to(dev)
    d_out = torch.zeros(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    got = []
    for k in (0, 1, 0):  # consecutive calls, the scratch array keeps the last call's data
        st = _noalloc(lib, mode, case, d_us, d_mov, mats[k], d_out, stream)
        assert st == 0, lib.lc2_last_error().decode()
        torch.cuda.synchronize()
        v = float(d_out.item())
        assert abs(v / ref[k] - 1.0) < REL, (k, v, ref[k])
        assert abs(v / orc[k] - 1.0) < REL, (k, v, orc[k])
        got.append(v)
    assert got[0] == got[2]


def test_noalloc_rejects_grids_over_the_limit():
    import torch

    lib = capi.load()
    big = synth.Case("3D", synth.Geometry((256, 256, 17), (1, 1, 1), (0, 0, 0)), None,
                     synth.Geometry((8, 8, 8), (1, 1, 1), (0, 0, 0)), None, [1, 1, 1], 2)
    d = torch.zeros(8, device="cuda:0")
    out = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    st = _noalloc(lib, "3D", big, d, d, np.eye(4, dtype=np.float32), out, 0)
    assert st == 6  # LC2_ERR_UNSUPPORTED
    assert b"LC2_NOALLOC_MAX_VOXELS" in lib.lc2_last_error()


def test_noalloc_refuses_a_capturing_stream():
    """Every call blocks on a read-back of the input maxima, so on a stream
    that is being captured into a CUDA graph it returns LC2_ERR_UNSUPPORTED
    before enqueuing anything, and the caller's capture stays valid."""
    import torch

    lib = capi.load()
    case = _case("2D")
    dev = torch.device("cuda:0")
    d_us = torch.from_numpy(np.ascontiguousarray(case.fixed, np.float32)).to(dev)
    d_mov = torch.from_numpy(np.ascontiguousarray(case.moving, np.float32)).to(dev)
    d_out = torch.zeros(1, dtype=torch.float64, device=dev)
    side = torch.cuda.Stream(dev)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        st = _noalloc(lib, "2D", case, d_us, d_mov, case.true_mat, d_out, side.cuda_stream)
        d_out.add_(1.0)  # the capture is still usable after the refused call
    assert st == 6, st
    assert b"capturing" in lib.lc2_last_error()
    g.replay()
    torch.cuda.synchronize()
    assert float(d_out.item()) == 1.0
