"""Cundall-Strack contacts (forces/cundall_strack.py:22-242) on the device, through the
C ABI, against the oracle's restatement.

The law is velocity- and spin-dependent and exerts torques, so the engine runs
it as two kernels per step with the rotational integrator every step.  No
reference test covers the law; the oracle is pinned by hand-derived closed
forms in test_oracle_pins.py.  Bars: force and torque <= 1e-5 floored relative
error from identical inputs; 50-step rollouts with rotation <= 1e-4 in
position; pair energy to float32 round-off.
"""

from __future__ import annotations

import numpy as np
import pytest

import jaxdem_gb300 as jdem
from jaxdem_gb300 import workloads as W
from jaxdem_gb300._lib import Engine
from oracle import dem_ref as R
from tests.helpers import force_err, min_image_diff, osystem, ostate

pytestmark = pytest.mark.gpu

F32 = np.float32
MATS = dict(young=[1e3, 3e3], poisson=[0.25, 0.3], e=[0.6, 0.8], mu=[0.4, 0.3], mu_r=[0.05, 0.1])
BETA, PROPS = R.cs_tables(**MATS)


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def periodic(N=2000, seed=51, dim=3, phi=0.55):
    rng = np.random.Generator(np.random.PCG64(seed))
    return W.periodic_system("cs", rng, N, dim, rng.choice([0.5, 0.6], size=N), phi, 0.3, 1e-3, 50)


def cases():
    p3 = periodic()
    p2 = periodic(dim=2, phi=0.7, seed=52)
    refl = W.c3(N=2000, seed=53)
    refl.vel = np.random.default_rng(1).normal(0, 0.5, size=refl.vel.shape).astype(F32)
    free = periodic(N=1200, seed=54, phi=0.35)
    free.domain = "free"
    return {"periodic3d": p3, "periodic2d": p2, "reflect2d": refl, "free3d": free}


def spins(w, seed=3, scale=2.0):
    ad = 3 if w.dim == 3 else 1
    return np.random.default_rng(seed).normal(0, scale, (w.N, ad)).astype(F32)


def materials(w, seed=5):
    return np.random.default_rng(seed).integers(0, 2, w.N).astype(np.int32)


def engine(w, rotation="verletspiral", skin=0.1):
    d = w.desc()
    d["rotation"] = rotation
    return Engine(w.dim, [d], BETA, skin=skin, force_law="cundallstrack", material_props=PROPS)


def osys(w, rotation="verletspiral"):
    sy = osystem(w, young=BETA, rotation=rotation)
    sy.force_law, sy.mat_props = "cundallstrack", PROPS
    return sy


@pytest.mark.parametrize("case", ["periodic3d", "periodic2d", "reflect2d", "free3d"])
def test_cs_force_and_torque_match_oracle(case):
    w = cases()[case]
    ang, mat = spins(w), materials(w)
    st = ostate(w, ang_vel=ang, mat_id=mat)
    sy = osys(w)
    f64, t64 = R.cell_list_force(st, sy, sum_dtype=np.float64)
    eng = engine(w)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel, ang_vel=ang, mat_id=mat)
        eng.compute_force()
        out = eng.download()
        e_dev = eng.energy()
    finally:
        eng.close()
    assert np.abs(t64).max() > 0
    assert force_err(out["force"], f64) <= 1e-5
    assert force_err(out["torque"], t64) <= 1e-5
    pe = R.cell_list_energy(st, sy, sum_dtype=np.float64)
    assert abs(e_dev[0] - pe) <= 1e-5 * abs(pe)


@pytest.mark.parametrize("case,rotation", [("periodic3d", "verletspiral"), ("periodic2d", "verletspiral"),
                                           ("reflect2d", "verletspiral"), ("free3d", "verletspiral"),
                                           ("periodic3d", "spiral")])
def test_cs_rollout_matches_oracle(case, rotation, steps=50):
    w = cases()[case]
    ang, mat = spins(w), materials(w)
    st = ostate(w, ang_vel=ang, mat_id=mat)
    sy = osys(w, rotation=rotation)
    st, sy = R.step(st, sy, steps, sum_dtype=np.float64)
    eng = engine(w, rotation=rotation)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel, ang_vel=ang, mat_id=mat)
        eng.step(steps)
        out = eng.download()
        box, anc = eng.domain_state()
    finally:
        eng.close()
    per_box = w.box_size if w.domain == "periodic" else None
    assert min_image_diff(out["pos_c"], st.pos_c, per_box) <= 1e-4
    assert np.abs(out["vel"] - st.vel).max() <= 1e-3 * max(1.0, np.abs(st.vel).max())
    assert np.abs(out["ang_vel"] - st.ang_vel).max() <= 1e-3 * max(1.0, np.abs(st.ang_vel).max())
    q = np.concatenate([st.q.w, st.q.xyz], 1) if hasattr(st.q, "w") else st.q
    assert np.abs(out["q"] - q).max() <= 1e-4
    assert force_err(out["force"], st.force) <= 1e-3
    assert force_err(out["torque"], st.torque) <= 1e-3
    if w.domain == "free":
        assert np.allclose(box[0], sy.box_size, rtol=1e-5, atol=1e-5)


def test_cs_dissipates_energy():
    """With e < 1 and friction the total energy of a periodic packing only decreases."""
    w = periodic(N=3000, seed=55)
    eng = engine(w)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel, ang_vel=spins(w))
        e = [float(np.sum(eng.energy()))]
        for _ in range(5):
            eng.step(40)
            e.append(float(np.sum(eng.energy())))
    finally:
        eng.close()
    assert all(b < a for a, b in zip(e, e[1:])), e


def test_cs_through_the_public_api():
    """System.create(force_model_type="cundallstrack") with elasticfrict materials; the
    rollout streams the moving rotational state."""
    w = periodic(N=1000, seed=56)
    mats = [jdem.Material.create("elasticfrict", young=MATS["young"][k], poisson=MATS["poisson"][k],
                                 e=MATS["e"][k], mu=MATS["mu"][k], mu_r=MATS["mu_r"][k]) for k in range(2)]
    table = jdem.MaterialTable.from_materials(mats)
    mat = materials(w)
    st = jdem.State.create(pos=w.pos, vel=w.vel, rad=w.rad, mat_table=table, mat_id=mat)
    st.ang_vel = spins(w)
    sy = jdem.System.create(state=st, collider_type="CellList", domain_type="periodic", mat_table=table,
                            dt=1e-3, force_model_type="cundallstrack",
                            domain_kw=dict(box_size=w.box_size, anchor=w.anchor))
    fs, _, (frames, _) = jdem.System.trajectory_rollout(st, sy, n=3, stride=5)
    ost = R.make_state(w.pos, vel=w.vel, rad=w.rad, mass=st.mass, mat_id=mat, ang_vel=st.ang_vel)
    osy = osys(w)
    ost, _ = R.step(ost, osy, 15, sum_dtype=np.float64)
    assert min_image_diff(fs.pos_c, ost.pos_c, w.box_size) <= 1e-5
    assert np.abs(fs.ang_vel - ost.ang_vel).max() <= 1e-4 * max(1.0, np.abs(ost.ang_vel).max())
    assert not np.array_equal(frames.ang_vel[0], frames.ang_vel[-1])
    assert np.array_equal(frames.ang_vel[-1], fs.ang_vel)
