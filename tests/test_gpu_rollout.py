"""Trajectory frames streamed from the device (``jdem_rollout``) against the same
engine stepped stride by stride and read back with ``jdem_download``.

``System.trajectory_rollout`` (system.py:606-699) scans ``System.step(n=k)`` and
saves ``save_fn(state, system)`` after each stride; a stride of 0 saves the
current state again.  The engine's steps are deterministic (the slot order is
sorted by system, cell and original index), so every streamed frame must equal
the stepped-and-downloaded state bit for bit, whichever copy path carried it:
page-locked destinations, pageable destinations through the staging ring, or
frames kept in device memory.
"""

from __future__ import annotations

import numpy as np
import pytest

import jaxdem_gb300 as jdem
from jaxdem_gb300 import workloads as W
from jaxdem_gb300._lib import Engine, JdemError, host_register, host_unregister
from tests.helpers import min_image_diff

pytestmark = pytest.mark.gpu

F32 = np.float32
K = np.array([[1e3]], F32)
FIELDS = ("pos_c", "vel", "force", "q", "ang_vel", "torque")


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def periodic(N=4096, seed=11, dim=3, phi=0.45):
    rng = np.random.Generator(np.random.PCG64(seed))
    return W.periodic_system("t", rng, N, dim, rng.choice([0.5, 0.6], size=N), phi, 0.2, 1e-3, 10)


def engine(ws, rotation="", skin=0.1):
    descs = []
    for w in ws:
        d = w.desc()
        d["rotation"] = rotation
        descs.append(d)
    return Engine(ws[0].dim, descs, K, skin=skin)


def upload(eng, ws, ang=None):
    cat = lambda k: np.concatenate([getattr(w, k) for w in ws])
    eng.upload(pos=cat("pos"), rad=cat("rad"), mass=cat("mass"), vel=cat("vel"), ang_vel=ang)


def stepped(eng, ws, strides, ang=None):
    """Reference frames: step each stride, then download."""
    upload(eng, ws, ang)
    frames = {k: [] for k in FIELDS}
    boxes, anchors = [], []
    for k in strides:
        eng.step(int(k))
        out = eng.download()
        for f in FIELDS:
            frames[f].append(out[f])
        b, a = eng.domain_state()
        boxes.append(b)
        anchors.append(a)
    res = {k: np.stack(v) for k, v in frames.items()}
    res["box"], res["anchor"] = np.stack(boxes), np.stack(anchors)
    return res


STRIDES = np.array([0, 3, 7, 0, 5, 1, 12, 2], np.int64)


@pytest.mark.parametrize("ring", [0, 1, 2, 16])
def test_streamed_frames_equal_stepped_frames(ring):
    w = periodic()
    eng = engine([w])
    try:
        ref = stepped(eng, [w], STRIDES)
        upload(eng, [w])
        got = eng.rollout(STRIDES, ring=ring)
        for k in FIELDS + ("box", "anchor"):
            assert np.array_equal(got[k], ref[k]), k
        # the handle ends where the last frame is
        assert np.array_equal(eng.download()["pos_c"], got["pos_c"][-1])
    finally:
        eng.close()


def test_page_locked_and_device_destinations():
    torch = pytest.importorskip("torch")
    w = periodic(N=3000, seed=12)
    T, P = len(STRIDES), w.N
    eng = engine([w])
    try:
        ref = stepped(eng, [w], STRIDES)
        # page-locked host destinations: written by the copy engine directly
        pinned = {k: np.empty((T, P, 3), F32) for k in ("pos_c", "vel", "force")}
        for a in pinned.values():
            host_register(a)
        try:
            upload(eng, [w])
            got = eng.rollout(STRIDES, fields=("pos_c", "vel", "force"), out=pinned)
            for k in pinned:
                assert got[k] is pinned[k]
                assert np.array_equal(pinned[k], ref[k]), k
        finally:
            for a in pinned.values():
                host_unregister(a)
        # device destinations: frames stay in HBM
        dev = {k: torch.empty((T, P, 3), dtype=torch.float32, device="cuda") for k in ("pos_c", "force")}
        upload(eng, [w])
        eng.rollout(STRIDES, fields=("pos_c", "force"), out=dev)
        torch.cuda.synchronize()
        for k in dev:
            assert np.array_equal(dev[k].cpu().numpy(), ref[k]), k
    finally:
        eng.close()


def test_free_domain_frame_boxes():
    """FreeDomain.apply (free.py:40-63): every frame carries the bounding box of its
    last step; a stride of 0 repeats the previous frame's box."""
    w = periodic(N=1500, seed=13, phi=0.3)
    w.domain = "free"
    eng = engine([w])
    try:
        ref = stepped(eng, [w], STRIDES)
        upload(eng, [w])
        got = eng.rollout(STRIDES)
        for k in FIELDS + ("box", "anchor"):
            assert np.array_equal(got[k], ref[k]), k
        assert not np.array_equal(got["box"][1], got["box"][-1])
    finally:
        eng.close()


def test_rotating_spheres_stream_orientation():
    """With nonzero angular velocity the spiral integrator moves q: the
    rotational fields are streamed per frame."""
    w = periodic(N=2000, seed=14, dim=3)
    ang = np.random.default_rng(3).normal(0, 1.0, (w.N, 3)).astype(F32)
    eng = engine([w], rotation="verletspiral")
    try:
        ref = stepped(eng, [w], STRIDES, ang=ang)
        upload(eng, [w], ang=ang)
        got = eng.rollout(STRIDES, ring=2)
        for k in FIELDS:
            assert np.array_equal(got[k], ref[k]), k
        assert not np.array_equal(got["q"][1], got["q"][-1])
    finally:
        eng.close()


def test_several_systems_and_2d():
    ws = [periodic(N=900, seed=s, dim=2, phi=0.6) for s in (21, 22, 23)]
    eng = engine(ws)
    try:
        ref = stepped(eng, ws, STRIDES)
        upload(eng, ws)
        got = eng.rollout(STRIDES, ring=3)
        for k in FIELDS + ("box", "anchor"):
            assert np.array_equal(got[k], ref[k]), k
        assert got["pos_c"].shape == (len(STRIDES), 2700, 2)
        assert got["box"].shape == (len(STRIDES), 3, 2)
    finally:
        eng.close()


def test_rollout_edge_cases():
    w = periodic(N=600, seed=15)
    eng = engine([w])
    try:
        upload(eng, [w])
        # no frames: nothing runs
        got = eng.rollout(np.zeros(0, np.int64))
        assert got["pos_c"].shape == (0, 600, 3)
        assert eng.stats()["steps"] == 0
        # zero strides only: the current state, repeated
        got = eng.rollout(np.zeros(5, np.int64), ring=2)
        assert all(np.array_equal(got["pos_c"][t], w.pos) for t in range(5))
        with pytest.raises(JdemError):
            eng.rollout(np.array([2, -1], np.int64))
        with pytest.raises(ValueError):
            eng.rollout(np.array([1], np.int64), out={"pos_c": np.empty((2, 600, 3), F32)})
    finally:
        eng.close()


def test_trajectory_rollout_api_uses_streamed_frames():
    """The public API: default save_fn stacks (state, system) per frame; a custom
    save_fn sees every frame; free-domain systems carry their per-frame boxes."""
    rng = np.random.Generator(np.random.PCG64(5))
    w = W.periodic_system("t", rng, 800, 3, rng.choice([0.5, 0.6], size=800), 0.3, 0.2, 1e-3, 10)
    mats = [jdem.Material.create("elastic", young=1e3, poisson=0.3, density=1.0)]
    table = jdem.MaterialTable.from_materials(mats)
    st = jdem.State.create(pos=w.pos, vel=w.vel, rad=w.rad, mat_table=table)
    sy = jdem.System.create(state=st, collider_type="CellList", domain_type="free", mat_table=table, dt=1e-3)
    fs, fy, (states, systems) = jdem.System.trajectory_rollout(st, sy, strides=STRIDES)
    assert states.pos_c.shape == (len(STRIDES), 800, 3)
    assert np.array_equal(systems.step_count, np.cumsum(STRIDES))
    # stepping call by call re-uploads (and re-sorts) every time, which may change
    # the summation order of a few contact sums: equal to float32 round-off
    cur_s, cur_y = st, sy
    for t, k in enumerate(STRIDES):
        cur_s, cur_y = jdem.System.step(cur_s, cur_y, n=int(k))
        assert min_image_diff(states.pos_c[t], cur_s.pos_c) <= 1e-5
        assert np.abs(states.vel[t] - cur_s.vel).max() <= 1e-5
        assert np.allclose(systems.domain.box_size[t], cur_y.domain.box_size, rtol=1e-6, atol=1e-5)
        assert np.allclose(systems.domain.anchor[t], cur_y.domain.anchor, rtol=1e-6, atol=1e-5)
        assert systems.time[t] == cur_y.time
    assert np.array_equal(fs.pos_c, states.pos_c[-1]) and fy.step_count == cur_y.step_count
    _, _, kin = jdem.System.trajectory_rollout(st, sy, n=3, stride=4,
                                               save_fn=lambda s, y: (s.vel, y.time))
    assert kin[0].shape == (3, 800, 3) and kin[1].shape == (3,)
    _, _, none = jdem.System.trajectory_rollout(st, sy, n=0)
    assert none[0].pos_c.shape == (0, 800, 3)
