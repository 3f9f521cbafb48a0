"""The request loop on the GPU: a mixed stream of 2D, 3D and 2D-to-3D
registrations, in both HighResolutionModality settings, submitted at random
times runs concurrently (each on its own context and stream), and every
result equals, bit for bit, the same registration run alone."""
import time

import numpy as np
import pytest

from lc2registration_gb300 import capi, synth
from lc2registration_gb300.geometry import Geometry
from tests.helpers import make_context

pytestmark = pytest.mark.gpu


def _reg(case):
    c = case.fixed_geom.center()
    if case.mode == "2D":
        return dict(initial=[0, 0, 0, 1, 1, 0], lower=[-10, -10, -8, 0.9, 0.9, -0.06],
                    upper=[10, 10, 8, 1.1, 1.1, 0.06], center=c, direct_entries=["translation"],
                    direct_maxeval=40, rounds=[(["translation", "rotation"], 1e-4)])
    lo = [-10, -10, -10, -8, -8, -8, 0.9, 0.9, 0.9, -0.05, -0.05, -0.05]
    hi = [10, 10, 10, 8, 8, 8, 1.1, 1.1, 1.1, 0.05, 0.05, 0.05]
    return dict(initial=[0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0], lower=lo, upper=hi, center=c,
                direct_entries=["translation"], direct_maxeval=40,
                rounds=[(["translation", "rotation"], 1e-3)])


def _fixed_roles(case):
    """HighResolutionModality: Fixed: the MR is the fixed image, the
    ultrasound is warped."""
    nd = 2 if case.mode == "2D" else 3
    return synth.Case(case.mode, case.moving_geom, case.moving, case.fixed_geom, case.fixed,
                      list(case.moving_geom.spacing[:nd]), case.r, hr_moving=False,
                      true_params={}, true_mat=None)


def _mix():
    cases = [synth.case_2d(seed=s, size=96, r=3) for s in (11, 12, 13)]
    cases += [synth.case_3d(seed=s, mr_size=40, us_size=32, r=2, blobs=6) for s in (14, 15)]
    cases += [_fixed_roles(synth.case_2d(seed=18, size=96, r=3)),
              _fixed_roles(synth.case_3d(seed=19, mr_size=40, us_size=32, r=2, blobs=6))]
    mr = synth.mr_phantom((48, 48, 48), 8, 1.5, seed=16)
    mg = Geometry((48, 48, 48), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0))
    cases += synth.frame_stack(mr, mg, 2, seed=17, sides=(40, 56), spacing=0.5, r=3)
    return cases


def test_mixed_stream_equals_alone():
    cases = _mix()
    alone = [capi.register(make_context(c), **_reg(c)) for c in cases]
    srv = capi.Server(budget_bytes=2 << 30, max_active=4)
    rng = np.random.default_rng(5)
    tickets = []
    for i in rng.permutation(len(cases)):
        c = cases[i]
        cfg = capi.make_config(c.mode, c.fixed_geom, c.moving_geom, c.virt_spacing, c.r,
                               c.hr_moving)
        tickets.append((i, srv.submit(cfg, c.fixed, c.moving, **_reg(c))))
        time.sleep(rng.exponential(0.01))
    for i, t in tickets:
        r = srv.poll(t)
        assert r["status"] == 0, r["message"]
        n = 6 if cases[i].mode == "2D" else 12
        np.testing.assert_array_equal(r["params"][:n], alone[i]["params"])
        assert r["lc2"] == alone[i]["lc2"]
        assert r["evaluations"] == alone[i]["evaluations"]
    st = srv.stats()
    assert st["completed"] == len(cases) and st["failed"] == 0
    assert st["peak_active"] >= 2            # requests did overlap
    assert st["p99_ms"] >= st["p50_ms"] > 0
    srv.close()


def test_stack_request_equals_stack_registration():
    mr = synth.mr_phantom((48, 48, 48), 8, 1.5, seed=18)
    mg = Geometry((48, 48, 48), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0))
    frames = synth.frame_stack(mr, mg, 3, seed=19, sides=(40, 56), spacing=0.5, r=3)
    regs = [_reg(f) for f in frames]
    st = capi.Stack(mg, 3)
    st.set_moving(mr)
    for f in frames:
        st.add_frame(f.fixed_geom, f.virt_spacing, f.fixed)
    want, _ = st.register(list(range(3)), regs)
    srv = capi.Server(budget_bytes=2 << 30, max_active=2)
    c2 = synth.case_2d(seed=20, size=64, r=3)
    cfg = capi.make_config(c2.mode, c2.fixed_geom, c2.moving_geom, c2.virt_spacing, c2.r)
    t_other = srv.submit(cfg, c2.fixed, c2.moving, **_reg(c2))
    t = srv.submit_stack(mg, mr, 3, [(f.fixed_geom, f.fixed) for f in frames],
                         frames[0].virt_spacing, regs)
    got = srv.poll_stack(t)
    assert srv.poll(t_other)["status"] == 0
    for g, w in zip(got, want):
        assert g["status"] == 0, g["message"]
        np.testing.assert_array_equal(g["params"][:12], w["params"])
        assert g["lc2"] == w["lc2"]
    with pytest.raises(capi.LC2Error, match="unknown"):
        srv.poll_stack(t)
    srv.close()


def test_merger_equals_each_context_alone():
    """lc2_merger_evaluate: transforms of 2D contexts of different sizes (and,
    separately, 2D-to-3D frames of different sizes with their own volumes) in
    one launch give each context's own lc2_evaluate_batch values bit for bit."""
    rng = np.random.default_rng(8)
    m = capi.Merger()
    cases = [synth.case_2d(seed=s, size=sz, r=3) for s, sz in ((31, 64), (32, 96), (33, 72))]
    for group in (cases, None):
        if group is None:
            group = []
            for s, sides in ((34, (40,)), (35, (56,))):
                mr = synth.mr_phantom((40, 40, 40), 6, 1.5, seed=s)
                mg = Geometry((40, 40, 40), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0))
                group += synth.frame_stack(mr, mg, 1, seed=s + 1, sides=sides, spacing=0.5, r=3)
        ctxs = [make_context(c) for c in group]
        from tests.helpers import perturbed
        mats = [perturbed(c, rng, k) for c, k in zip(group, (5, 1, 3)[:len(group)])]
        got = m.evaluate(ctxs, mats)
        for c, mm, g in zip(ctxs, mats, got):
            np.testing.assert_array_equal(g, c.evaluate_batch(mm))
    assert m.launch_count() == 4  # list kernel + ratio per merged call
    m.close()


def test_concurrent_2d_requests_share_launches():
    """Six 2D registrations running at once: their optimizer steps are merged
    into shared launches, and each result equals the registration alone."""
    cases = [synth.case_2d(seed=s, size=sz, r=3) for s, sz in
             ((41, 64), (42, 80), (43, 64), (44, 96), (45, 72), (46, 64))]
    alone = [capi.register(make_context(c), **_reg(c)) for c in cases]
    srv = capi.Server(budget_bytes=2 << 30, max_active=len(cases), merge_window_us=2000)
    tickets = []
    for c in cases:
        cfg = capi.make_config(c.mode, c.fixed_geom, c.moving_geom, c.virt_spacing, c.r, True)
        tickets.append(srv.submit(cfg, c.fixed, c.moving, **_reg(c)))
    for t, a in zip(tickets, alone):
        r = srv.poll(t)
        assert r["status"] == 0, r["message"]
        np.testing.assert_array_equal(r["params"][:6], a["params"])
        assert r["lc2"] == a["lc2"] and r["evaluations"] == a["evaluations"]
    st = srv.stats()
    assert st["merged_launches"] > 0
    assert st["merged_steps"] > 1.5 * st["merged_launches"], st
    srv.close()
