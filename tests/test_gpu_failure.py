"""Failure detection on the GPU without a fault: every producer/consumer wait
of the warp-specialised kernel gives up after one second and reports
LC2_ERR_TIMEOUT through a device flag the host reads. lc2_wait_probe runs
that same bounded wait on a barrier nothing completes, so the wait runs out
by itself; the context must report the timeout once and then evaluate as
before, bit for bit, on both kernels."""
import time

import numpy as np
import pytest

from lc2registration_gb300 import capi, synth
from tests.helpers import make_context, perturbed

pytestmark = pytest.mark.gpu


def test_expired_wait_is_reported_and_context_stays_usable():
    case = synth.case_3d(seed=41, mr_size=40, us_size=32, r=2, blobs=5)
    ctx = make_context(case, "f16")
    mats = perturbed(case, np.random.default_rng(9), 5)
    # the warp-specialised kernel resamples in place: compare with that form
    ctx.set_option(capi.OPTION_PRESAMPLE, 0)
    before = ctx.evaluate_batch(mats)
    t0 = time.perf_counter()
    with pytest.raises(capi.LC2Error, match="LC2_ERR_TIMEOUT"):
        ctx.wait_probe()
    waited = time.perf_counter() - t0
    assert 0.9 < waited < 30.0, waited  # the one-second limit, not a hang
    # reported once: the flag is cleared, later calls succeed
    np.testing.assert_array_equal(ctx.evaluate_batch(mats), before)
    ctx.set_option(capi.OPTION_PIPELINE, 1)
    np.testing.assert_array_equal(ctx.evaluate_batch(mats), before)
    ctx.set_option(capi.OPTION_PIPELINE, 0)
    np.testing.assert_array_equal([ctx.evaluate(m) for m in mats[:2]], before[:2])


def _live():
    import ctypes
    lib = capi.load()
    b, n = ctypes.c_size_t(), ctypes.c_longlong()
    assert lib.lc2_debug_device_bytes(ctypes.byref(b), ctypes.byref(n)) == 0
    return b.value, n.value


def _sweep_failures(make, max_k=80):
    """Arms an injected out-of-memory at the k-th allocation for k = 1, 2, ...
    and runs make() until it needs fewer allocations than k. Each failing run
    must raise LC2_ERR_OUT_OF_MEMORY and leave the library's device memory as
    it found it; returns how many allocations the call makes."""
    lib = capi.load()
    base = _live()
    try:
        for k in range(1, max_k + 1):
            lib.lc2_debug_fail_allocation(k)
            try:
                obj = make()
            except capi.LC2Error as e:
                assert e.status == 2, (k, e)  # LC2_ERR_OUT_OF_MEMORY
                assert _live() == base, (k, _live(), base)
                continue
            lib.lc2_debug_fail_allocation(0)
            obj.close()
            assert _live() == base
            return k - 1
    finally:
        lib.lc2_debug_fail_allocation(0)
    raise AssertionError("the call kept allocating")


@pytest.mark.parametrize("mode", ["2D", "3D", "3D_fixed"])
def test_injected_out_of_memory_in_create_and_upload_is_clean(mode):
    """Failure injection on the host (lc2_debug_fail_allocation): every device
    or pinned allocation of lc2_create + lc2_set_images + a first batch is made
    to fail in turn; each failure returns LC2_ERR_OUT_OF_MEMORY and frees what
    the call had taken, and the next attempt works."""
    if mode == "2D":
        case = synth.case_2d(seed=51, size=48, r=3)
    else:
        case = synth.case_3d(seed=52, mr_size=32, us_size=24, r=2, blobs=4)
    hr = mode != "3D_fixed"
    mats = perturbed(case, np.random.default_rng(1), 100)

    def make():
        if not hr:
            c = synth.Case(case.mode, case.moving_geom, case.moving, case.fixed_geom, case.fixed,
                           [1.0, 1.0, 1.0], case.r, hr_moving=False)
        else:
            c = case
        ctx = capi.Context(c.mode, c.fixed_geom, c.moving_geom, c.virt_spacing, c.r, hr)
        try:
            ctx.set_images(c.fixed, c.moving)
            ctx.evaluate_batch(mats)  # grows the transform buffers past 64
        except Exception:
            ctx.close()
            raise
        return ctx

    n = _sweep_failures(make)
    assert n >= 5


def test_injected_out_of_memory_in_stack_and_server():
    from lc2registration_gb300.geometry import Geometry

    mr = synth.mr_phantom((40, 40, 40), 6, 1.5, seed=53)
    mg = Geometry((40, 40, 40), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0))
    frames = synth.frame_stack(mr, mg, 2, seed=54, sides=(40, 56), spacing=0.5, r=3)

    def make_stack():
        st = capi.Stack(mg, 3)
        try:
            st.set_moving(mr)
            for f in frames:
                st.add_frame(f.fixed_geom, f.virt_spacing, f.fixed)
            st.evaluate(np.array([0, 1], dtype=np.int32),
                        np.stack([frames[0].true_mat, frames[1].true_mat]))
        except Exception:
            st.close()
            raise
        return st

    assert _sweep_failures(make_stack) >= 5

    # a request whose allocations fail completes with the status; the server
    # goes on with the next request
    lib = capi.load()
    case = synth.case_2d(seed=55, size=48, r=3)
    cfg = capi.make_config(case.mode, case.fixed_geom, case.moving_geom, case.virt_spacing,
                           case.r)
    reg = dict(initial=[0, 0, 0, 1, 1, 0], lower=[-5, -5, -5, 0.9, 0.9, -0.05],
               upper=[5, 5, 5, 1.1, 1.1, 0.05], center=case.fixed_geom.center(),
               rounds=[(["translation"], 1e-3)])
    srv = capi.Server(budget_bytes=1 << 30, max_active=1)
    base = _live()
    lib.lc2_debug_fail_allocation(1)
    bad = srv.poll(srv.submit(cfg, case.fixed, case.moving, **reg))
    lib.lc2_debug_fail_allocation(0)
    assert bad["status"] == 2, bad
    good = srv.poll(srv.submit(cfg, case.fixed, case.moving, **reg))
    assert good["status"] == 0, good["message"]
    st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == 1
    srv.close()
    assert _live()[0] <= base[0] + (64 << 20)  # the merge group's buffers may stay
