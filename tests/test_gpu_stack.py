"""2D-to-3D frame stacks (lc2_stack_*): frames of uneven sizes and their
candidate poses evaluated in one work-list launch must give, bit for bit,
what a standalone 2D-to-3D context of each frame gives, and match the FP64
oracle within 1e-5."""
import numpy as np
import pytest

from lc2registration_gb300 import capi, synth
from lc2registration_gb300.geometry import Geometry
from tests.helpers import make_context, oracle_eval, perturbed

pytestmark = pytest.mark.gpu


def _frames(n, seed, sides=(24, 40, 56, 72), r=3):
    mr = synth.mr_phantom((48, 48, 48), 8, 1.5, seed=seed)
    mg = Geometry((48, 48, 48), (1.0, 1.0, 1.0), (0.0, 0.0, 0.0))
    return mr, mg, synth.frame_stack(mr, mg, n, seed=seed + 1, sides=sides, spacing=0.5, r=r)


def _stack(mr, mg, frames, r, storage="f32"):
    st = capi.Stack(mg, r, storage)
    st.set_moving(mr)
    for i, f in enumerate(frames):
        assert st.add_frame(f.fixed_geom, f.virt_spacing, f.fixed) == i
    return st


def _requests(frames, per_frame, rng):
    ids, mats = [], []
    for i, f in enumerate(frames):
        for m in perturbed(f, rng, per_frame):
            ids.append(i)
            mats.append(m)
    order = rng.permutation(len(ids))  # interleave the frames
    return np.array(ids)[order], np.stack(mats)[order]


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_stack_equals_standalone_contexts(storage):
    mr, mg, frames = _frames(5, seed=40)
    assert len({f.fixed_geom.dim[0] for f in frames}) > 1, "frames should differ in size"
    st = _stack(mr, mg, frames, 3, storage)
    ids, mats = _requests(frames, 6, np.random.default_rng(0))
    got = st.evaluate(ids, mats)
    ctxs = [make_context(f, storage) for f in frames]
    want = np.array([ctxs[i].evaluate(m) for i, m in zip(ids, mats)])
    np.testing.assert_array_equal(got, want)
    # the frame's own context inside the stack agrees too
    fc = st.frame_context(int(ids[0]))
    assert fc.evaluate(mats[0]) == got[0]
    assert np.all(got > 0.0)


def test_stack_matches_oracle_and_truth():
    mr, mg, frames = _frames(4, seed=41)
    st = _stack(mr, mg, frames, 3)
    ids, mats = _requests(frames, 3, np.random.default_rng(1))
    ids = np.concatenate([ids, np.arange(len(frames))])
    mats = np.concatenate([mats, np.stack([f.true_mat for f in frames])])
    got = st.evaluate(ids, mats)
    for i, m, g in zip(ids, mats, got):
        ref = oracle_eval(frames[i], m)
        assert abs(g / ref - 1) < 1e-5, (i, g, ref)
    # the generating pose scores higher than the perturbed ones of its frame
    for i in range(len(frames)):
        assert got[len(got) - len(frames) + i] >= got[:-len(frames)][ids[:-len(frames)] == i].max()


def test_stack_graph_replay_and_layouts():
    mr, mg, frames = _frames(3, seed=42, sides=(24, 40), r=2)
    st = _stack(mr, mg, frames, 2)
    rng = np.random.default_rng(2)
    ctxs = [make_context(f) for f in frames]
    for rep in range(3):
        ids, mats = _requests(frames, 4, rng)     # same layout, new poses
        got = st.evaluate(ids, mats)
        want = np.array([ctxs[i].evaluate(m) for i, m in zip(ids, mats)])
        np.testing.assert_array_equal(got, want)
    assert st.graph_launches() == 3
    ids, mats = _requests(frames[:2], 5, rng)     # another layout
    np.testing.assert_array_equal(st.evaluate(ids, mats),
                                  [ctxs[i].evaluate(m) for i, m in zip(ids, mats)])
    st.set_graphs(False)
    np.testing.assert_array_equal(st.evaluate(ids, mats),
                                  [ctxs[i].evaluate(m) for i, m in zip(ids, mats)])
    assert st.graph_launches() == 4


@pytest.mark.parametrize("r", [1, 5, 12])
def test_stack_patch_radii(r):
    mr, mg, frames = _frames(2, seed=43, sides=(40, 56), r=r)
    st = _stack(mr, mg, frames, r)
    ids, mats = _requests(frames, 2, np.random.default_rng(3))
    got = st.evaluate(ids, mats)
    ctxs = [make_context(f) for f in frames]
    np.testing.assert_array_equal(got, [ctxs[i].evaluate(m) for i, m in zip(ids, mats)])


def test_stack_errors():
    mr, mg, frames = _frames(1, seed=44, sides=(24,))
    st = capi.Stack(mg, 3)
    f = frames[0]
    with pytest.raises(capi.LC2Error, match="NOT_READY"):
        st.add_frame(f.fixed_geom, f.virt_spacing, f.fixed)
    st.set_moving(mr)
    with pytest.raises(capi.LC2Error, match="already set"):
        st.set_moving(mr)
    bad = Geometry((24, 24, 2), f.fixed_geom.spacing, f.fixed_geom.origin)
    with pytest.raises(capi.LC2Error, match="INVALID_ARGUMENT"):
        st.add_frame(bad, f.virt_spacing, np.zeros(24 * 24 * 2, np.float32))
    fid = st.add_frame(f.fixed_geom, f.virt_spacing, f.fixed)
    with pytest.raises(capi.LC2Error, match="names frame"):
        st.evaluate([fid + 1], np.eye(4)[None])
    m = np.eye(4, dtype=np.float32)
    m[0, 0] = np.nan
    with pytest.raises(capi.LC2Error, match="NaN"):
        st.evaluate([fid], m[None])
    fc = st.frame_context(fid)
    with pytest.raises(capi.LC2Error, match="share"):
        fc.set_images(f.fixed, mr)
    assert st.evaluate([], np.zeros((0, 16))).shape == (0,)


def test_stack_register_equals_per_frame_registration():
    mr, mg, frames = _frames(4, seed=45, sides=(40, 56, 72))
    st = _stack(mr, mg, frames, 3)
    lo = [-6, -6, -6, -6, -6, -6, 0.95, 0.95, 0.95, -0.02, -0.02, -0.02]
    hi = [6, 6, 6, 6, 6, 6, 1.05, 1.05, 1.05, 0.02, 0.02, 0.02]
    regs = []
    for f in frames:
        regs.append(dict(initial=[0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0], lower=lo, upper=hi,
                         center=f.fixed_geom.center(), direct_entries=["translation"],
                         direct_maxeval=30, rounds=[(["translation", "rotation"], 1e-3)]))
    got, launches = st.register(list(range(len(frames))), regs)
    total_batches = 0
    for i, f in enumerate(frames):
        alone = capi.register(make_context(f), **regs[i])
        np.testing.assert_array_equal(got[i]["params"], alone["params"])
        assert got[i]["lc2"] == alone["lc2"]
        assert got[i]["evaluations"] == alone["evaluations"]
        total_batches += alone["launches"]
    # every round of optimizer steps of all frames went out as one stack call
    assert launches < total_batches
    # independent concurrent registrations on the frames' own contexts: same results
    st.set_option(capi.OPTION_STACK_BATCHING, 0)
    got2, launches2 = st.register(list(range(len(frames))), regs)
    assert launches2 == 0
    for a, b in zip(got, got2):
        np.testing.assert_array_equal(a["params"], b["params"])
        assert a["lc2"] == b["lc2"]
    with pytest.raises(capi.LC2Error, match="distinct"):
        st.register([0, 0], regs[:2])
