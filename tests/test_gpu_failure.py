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
