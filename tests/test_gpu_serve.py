"""Serving loop: continuous batching, admission, cancellation, and the
requirement that each request's result is the same alone and in the mix
(tolerance: 1e-5 position, minimum image)."""

from __future__ import annotations

import time

import numpy as np
import pytest

from jaxdem_gb300 import workloads as W
from jaxdem_gb300._lib import Engine, JdemError
from jaxdem_gb300.autotune import default_skin
from jaxdem_gb300.serve import Server
from tests.helpers import min_image_diff

pytestmark = pytest.mark.gpu

F32 = np.float32


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def req(N, seed, dim=3, phi=0.3, steps=200):
    rng = np.random.Generator(np.random.PCG64(seed))
    return W.periodic_system(f"r{seed}", rng, N, dim, rng.uniform(0.4, 0.6, N), phi, 0.05, 1e-3, steps)


def engine_result(w):
    eng = Engine(w.dim, [w.desc()], np.array([[W.K_SPRING]], F32), skin=default_skin(0.6))
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.step(w.steps)
        return eng.download()
    finally:
        eng.close()


def test_alone_equals_in_mix():
    a = req(1500, 1, steps=200)
    s = Server(3)
    try:
        ia = s.submit(a)
        s.drain(120)
        alone = s.result(ia)
    finally:
        s.close()
    mix = [req(500, 2, steps=50), a, req(3000, 3, phi=0.45, steps=120), req(256, 4, steps=400)]
    s = Server(3)
    try:
        ids = [s.submit(w) for w in mix]
        s.drain(120)
        res = [s.result(i) for i in ids]
        st = s.stats()
    finally:
        s.close()
    assert st["max_active"] >= 2 and st["repacks"] >= 3
    for w, r in zip(mix, res):
        assert r["info"]["state"] == "done" and r["info"]["steps"] == w.steps
    assert min_image_diff(res[1]["pos_c"], alone["pos_c"], a.box_size) <= 1e-5
    ref = engine_result(a)
    assert min_image_diff(alone["pos_c"], ref["pos_c"], a.box_size) <= 1e-5
    for w, r in zip(mix, res):
        assert min_image_diff(r["pos_c"], engine_result(w)["pos_c"], w.box_size) <= 1e-5


def test_cancellation_leaves_others_untouched():
    ws = [req(800, 10, dim=2, phi=0.5, steps=300), req(1200, 11, dim=2, phi=0.5, steps=300),
          req(600, 12, dim=2, phi=0.5, steps=150)]
    s = Server(2)
    try:
        ids = [s.submit(w) for w in ws]
        s.cancel(ids[1])
        s.drain(120)
        infos = [s.info(i) for i in ids]
        res = {i: s.result(i) for i, inf in zip(ids, infos) if inf["state"] == "done"}
    finally:
        s.close()
    assert infos[1]["state"] == "cancelled"
    for k in (0, 2):
        assert infos[k]["state"] == "done"
        assert min_image_diff(res[ids[k]]["pos_c"], engine_result(ws[k])["pos_c"], ws[k].box_size) <= 1e-5


def test_hbm_budget_limits_concurrency():
    ws = [req(1000, 20 + k, steps=60) for k in range(4)]
    s = Server(3, hbm_budget_gb=0.0012)  # room for one 1000-particle request (about 0.86 MB), not two
    try:
        ids = [s.submit(w) for w in ws]
        s.drain(120)
        st = s.stats()
        states = [s.info(i)["state"] for i in ids]
        with pytest.raises(JdemError):
            s.submit(req(5000, 30, steps=10))  # larger than the whole budget
    finally:
        s.close()
    assert st["max_active"] == 1 and states == ["done"] * 4


def test_bad_input_rejected_at_submit():
    w = req(100, 40, steps=10)
    w.pos[3, 1] = np.nan
    s = Server(3)
    try:
        with pytest.raises(JdemError):
            s.submit(w)
        ok = s.submit(req(100, 41, steps=10))
        s.drain(60)
        assert s.info(ok)["state"] == "done"
    finally:
        s.close()


def test_two_dimensions_served_concurrently():
    w2, w3 = req(2000, 50, dim=2, phi=0.6, steps=150), req(2000, 51, dim=3, phi=0.4, steps=150)
    s2, s3 = Server(2), Server(3)
    try:
        i2, i3 = s2.submit(w2), s3.submit(w3)
        s2.drain(120)
        s3.drain(120)
        r2, r3 = s2.result(i2), s3.result(i3)
    finally:
        s2.close()
        s3.close()
    assert min_image_diff(r2["pos_c"], engine_result(w2)["pos_c"], w2.box_size) <= 1e-5
    assert min_image_diff(r3["pos_c"], engine_result(w3)["pos_c"], w3.box_size) <= 1e-5


def test_release_while_batch_continues():
    """A finished request may be released while the rest of its batch still runs;
    the server keeps serving the others with the same results."""
    short, long_ = req(400, 60, steps=20), req(1500, 61, steps=300)
    s = Server(3, chunk_steps=10)
    try:
        i_long, i_short = s.submit(long_), s.submit(short)
        t0 = time.time()
        while s.info(i_short)["state"] != "done" and time.time() - t0 < 60:
            time.sleep(0.0005)
        assert s.info(i_short)["state"] == "done"
        s.result(i_short)
        s.release(i_short)
        with pytest.raises(JdemError):
            s.release(i_short)  # unknown id after release
        s.drain(120)
        r = s.result(i_long)
        st = s.stats()
    finally:
        s.close()
    assert st["completed"] == 2 and st["active"] == 0 and st["pending"] == 0
    assert min_image_diff(r["pos_c"], engine_result(long_)["pos_c"], long_.box_size) <= 1e-5


def _engine_alone(w, law, young, mat=None, ang=None, rotation="", props=None):
    d = w.desc()
    d["rotation"] = rotation
    eng = Engine(w.dim, [d], young, skin=default_skin(0.6), force_law=law, material_props=props)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel, mat_id=mat, ang_vel=ang)
        eng.step(w.steps)
        return eng.download()
    finally:
        eng.close()


@pytest.mark.parametrize("dim", [3, 2])
def test_hertz_materials_rotation_alone_equals_in_mix_and_engine(dim):
    """A Hertz server with two materials: a rotating request (VV-spiral in 3D, spiral in
    2D, random spins) and a two-material request give the same state alone, in a mix with
    other requests, and on a standalone engine handle (positions 1e-5, q and spin 2e-6)."""
    from oracle import dem_ref as R

    k43 = np.asarray(R.hertz_constant(np.array([1e3, 3e3]), np.array([0.3, 0.25])), F32)
    rot = "verletspiral" if dim == 3 else "spiral"
    ad = 3 if dim == 3 else 1
    rng = np.random.default_rng(50 + dim)
    a = req(1200, 11 + dim, dim=dim, phi=0.45, steps=150)
    a_mat = rng.integers(0, 2, a.N).astype(np.int32)
    a_ang = rng.normal(0, 2.0, (a.N, ad)).astype(F32)
    b = req(900, 21 + dim, dim=dim, phi=0.5, steps=90)
    b_mat = rng.integers(0, 2, b.N).astype(np.int32)

    def serve(items):
        s = Server(dim, force_law="hertz", young_eff=k43)
        try:
            ids = [s.submit(w, mat_id=m, ang_vel=g, rotation=r) for w, m, g, r in items]
            s.drain(120)
            return [s.result(i) for i in ids]
        finally:
            s.close()

    alone_a = serve([(a, a_mat, a_ang, rot)])[0]
    mix = serve([(req(400, 31, dim=dim, steps=40), None, None, ""), (a, a_mat, a_ang, rot),
                 (b, b_mat, None, ""), (req(2500, 32, dim=dim, phi=0.35, steps=200), None, None, "")])
    ref_a = _engine_alone(a, "hertz", k43, a_mat, a_ang, rot)
    ref_b = _engine_alone(b, "hertz", k43, b_mat)
    for got in (alone_a, mix[1]):
        assert got["info"]["state"] == "done"
        assert min_image_diff(got["pos_c"], ref_a["pos_c"], a.box_size) <= 1e-5
        assert np.allclose(got["q"], ref_a["q"], atol=2e-6)
        assert np.allclose(got["ang_vel"], ref_a["ang_vel"], atol=2e-6)
    assert not np.allclose(mix[1]["q"][:, 0], 1.0), "the spins should have rotated the spheres"
    assert min_image_diff(mix[2]["pos_c"], ref_b["pos_c"], b.box_size) <= 1e-5
    assert np.allclose(mix[2]["q"], np.array([1, 0, 0, 0], F32))


@pytest.mark.parametrize("dim", [3, 2])
def test_cundall_strack_alone_equals_in_mix_and_engine(dim):
    """A Cundall-Strack server (two elasticfrict materials, rolling friction): a spinning
    request gives the same state alone, in a mix whose repacks move it between epochs (its
    last torque travels with it: the next half-kick reads it), and on a standalone engine
    handle (positions 1e-5, q and spin 1e-5)."""
    from oracle import dem_ref as R

    beta, props = R.cs_tables(young=[1e3, 3e3], poisson=[0.25, 0.3], e=[0.6, 0.8], mu=[0.4, 0.3],
                              mu_r=[0.05, 0.1])
    rot = "verletspiral" if dim == 3 else "spiral"
    ad = 3 if dim == 3 else 1
    rng = np.random.default_rng(70 + dim)
    a = req(1200, 41 + dim, dim=dim, phi=0.45, steps=130)
    a_mat = rng.integers(0, 2, a.N).astype(np.int32)
    a_ang = rng.normal(0, 2.0, (a.N, ad)).astype(F32)

    def serve(items):
        s = Server(dim, force_law="cundallstrack", young_eff=beta, material_props=props, chunk_steps=20)
        try:
            ids = [s.submit(w, mat_id=m, ang_vel=g, rotation=r) for w, m, g, r in items]
            s.drain(120)
            return [s.result(i) for i in ids]
        finally:
            s.close()

    alone = serve([(a, a_mat, a_ang, rot)])[0]
    mix = serve([(req(400, 51, dim=dim, steps=30), None, None, ""), (a, a_mat, a_ang, rot),
                 (req(2000, 52, dim=dim, phi=0.35, steps=70), None, None, "")])
    ref = _engine_alone(a, "cundallstrack", beta, a_mat, a_ang, rot, props=props)
    for got in (alone, mix[1]):
        assert got["info"]["state"] == "done"
        assert min_image_diff(got["pos_c"], ref["pos_c"], a.box_size) <= 1e-5
        assert np.allclose(got["vel"], ref["vel"], atol=1e-5 * max(1.0, np.abs(ref["vel"]).max()))
        assert np.allclose(got["q"], ref["q"], atol=1e-5)
        assert np.allclose(got["ang_vel"], ref["ang_vel"], atol=1e-5 * max(1.0, np.abs(ref["ang_vel"]).max()))
    assert all(m["info"]["state"] == "done" for m in mix)
