"""Hertz normal contact (forces/hertz.py:22-170) on the device, through the C ABI,
against the oracle's restatement of the same law.

The reference has no test of this law, so the oracle is pinned by hand-derived
answers in test_oracle_pins.py (two spheres against the closed form, F = -dE/dd,
C against numpy).  Here the engine is held to the spring's tolerances:
floored relative force error <= 1e-5 from identical inputs, 100-step rollouts
<= 1e-4 in position, pair energy to float32 round-off, bit-exact contact sets.
"""

from __future__ import annotations

import numpy as np
import pytest

import jaxdem_gb300 as jdem
import oracle
from jaxdem_gb300 import workloads as W
from jaxdem_gb300._lib import Engine
from oracle import dem_ref as R
from tests.helpers import force_err, min_image_diff, osystem, ostate

pytestmark = pytest.mark.gpu

F32 = np.float32
YOUNG, POISSON = [1e3, 4e3], [0.3, 0.2]
K43 = R.hertz_constant(YOUNG, POISSON)


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def periodic(N=3000, seed=41, dim=3, phi=0.55, radii=(0.5, 0.7)):
    rng = np.random.Generator(np.random.PCG64(seed))
    return W.periodic_system("h", rng, N, dim, rng.choice(np.asarray(radii), size=N), phi, 0.1, 1e-3, 100)


def cases():
    p3 = periodic()
    p2 = periodic(dim=2, phi=0.7, seed=42)
    refl = W.c3(N=3000, seed=43)
    free = periodic(N=1500, seed=44, phi=0.3)
    free.domain = "free"
    return {"periodic3d": p3, "periodic2d": p2, "reflect2d": refl, "free3d": free}


def engine(w, mats=1, skin=0.1):
    table = K43[:mats, :mats] if mats > 1 else K43[:1, :1]
    return Engine(w.dim, [w.desc()], table, skin=skin, force_law="hertz")


def hertz_sys(w, mats=1):
    sy = osystem(w, young=K43[:mats, :mats])
    sy.force_law = "hertz"
    return sy


@pytest.mark.parametrize("case", ["periodic3d", "periodic2d", "reflect2d", "free3d"])
def test_hertz_force_matches_oracle(case):
    w = cases()[case]
    mat = np.random.default_rng(5).integers(0, 2, w.N).astype(np.int32)
    st = ostate(w, mat_id=mat)
    sy = hertz_sys(w, mats=2)
    ref64, _ = R.cell_list_force(st, sy, sum_dtype=np.float64)
    ref32, _ = R.cell_list_force(st, sy)
    eng = engine(w, mats=2)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel, mat_id=mat)
        eng.compute_force()
        out = eng.download()
        e_dev = eng.energy()
    finally:
        eng.close()
    assert np.abs(ref64).max() > 0
    assert force_err(out["force"], ref64) <= 1e-5
    assert force_err(out["force"], ref32) <= 1e-5
    pe = R.cell_list_energy(st, sy, sum_dtype=np.float64)
    assert abs(e_dev[0] - pe) <= 1e-5 * abs(pe)


@pytest.mark.parametrize("case", ["periodic3d", "periodic2d", "reflect2d", "free3d"])
def test_hertz_rollout_matches_oracle(case, steps=100):
    w = cases()[case]
    if case == "reflect2d":
        w.vel = np.random.default_rng(1).normal(0, 0.5, size=w.vel.shape).astype(F32)
    pos, vel, frc = w.pos.copy(), w.vel.copy(), np.zeros_like(w.pos)
    box_o, anc_o = oracle.c_step(w.dim, pos, vel, frc, w.rad, w.mass, domain=w.domain, box=w.box_size,
                                 anchor=w.anchor, dt=w.dt, steps=steps, cell_size=2 * float(w.rad.max()),
                                 gravity=w.gravity, restitution=w.restitution, acc64=True,
                                 young=K43[:1, :1], law="hertz")
    eng = engine(w)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.step(steps)
        out = eng.download()
        box, anc = eng.domain_state()
    finally:
        eng.close()
    per_box = w.box_size if w.domain == "periodic" else None
    assert min_image_diff(out["pos_c"], pos, per_box) <= 1e-4
    assert np.abs(out["vel"] - vel).max() <= 1e-3 * max(1.0, np.abs(vel).max())
    assert force_err(out["force"], frc) <= 1e-3
    if w.domain == "free":
        assert np.allclose(box[0], box_o, rtol=1e-5, atol=1e-5)
        assert np.allclose(anc[0], anc_o, rtol=1e-5, atol=1e-5)


def test_hertz_contact_set_equals_spring_contact_set():
    """Both laws act on the same pairs (delta > 0): the canonical contact set is the
    oracle's, bit for bit."""
    w = periodic(N=2500, seed=45)
    ref = R.contact_pairs(ostate(w), hertz_sys(w))
    eng = engine(w)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        got = eng.contacts()
    finally:
        eng.close()
    assert np.array_equal(got, ref)


def test_hertz_through_the_public_api():
    """System.create(force_model_type="hertz") with a young/poisson material table: one
    System.step against the oracle, and the host pair forces of get_pair_forces_and_ids."""
    w = periodic(N=1200, seed=46)
    mats = [jdem.Material.create("elastic", young=YOUNG[0], poisson=POISSON[0], density=1.0)]
    table = jdem.MaterialTable.from_materials(mats)
    st = jdem.State.create(pos=w.pos, vel=w.vel, rad=w.rad, mat_table=table)
    sy = jdem.System.create(state=st, collider_type="CellList", domain_type="periodic", mat_table=table,
                            dt=1e-3, force_model_type="hertz",
                            domain_kw=dict(box_size=w.box_size, anchor=w.anchor))
    st2, _ = jdem.System.step(st, sy, n=5)
    ost = R.make_state(w.pos, vel=w.vel, rad=w.rad, mass=st.mass)
    osy = hertz_sys(w)
    osy.rotation = ""
    ost, _ = R.step(ost, osy, 5, sum_dtype=np.float64)
    assert min_image_diff(st2.pos_c, ost.pos_c, w.box_size) <= 1e-5
    assert force_err(st2.force, ost.force) <= 1e-4
    _, _, ids, f = jdem.utils.get_pair_forces_and_ids(st2, sy, cutoff=1.5, max_neighbors=64)
    i, j = ids[:, 0], ids[:, 1]
    ok = j >= 0
    fr = R.hertz_pair(i[ok], j[ok], st2.pos_c, st2.rad, st2.mat_id, K43[:1, :1], osy)
    assert np.allclose(f[ok], fr, rtol=1e-5, atol=1e-5 * np.abs(fr).max())


def test_hertz_large_system_with_pruning_matches_oracle_and_full_list():
    """Above 32768 slots the fused list kernel runs the Hertz law with dynamic pruning and
    the branch-free list batches: step-0 forces against the oracle, and 60 steps with
    pruning equal to 60 steps on the full list bit for bit."""
    w = periodic(N=65536, seed=45)
    ost = ostate(w)
    st1, _ = R.step(ost, hertz_sys(w), 1, sum_dtype=np.float64)
    outs = []
    for ps in (0.0, -1.0):
        eng = Engine(w.dim, [w.desc()], K43[:1, :1], skin=0.3, force_law="hertz", prune_skin=ps)
        try:
            eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
            eng.step(1)
            first = eng.download()
            eng.step(59)
            outs.append((first, eng.download(), eng.stats()))
        finally:
            eng.close()
    (f_pr, pr, st_pr), (f_full, full, st_full) = outs
    assert force_err(f_pr["force"], st1.force) <= 1e-5
    assert min_image_diff(f_pr["pos_c"], st1.pos_c, w.box_size) <= 1e-5
    assert st_pr["prunes"] > 0 and st_full["prunes"] == 0
    for k in ("pos_c", "vel", "force"):
        assert np.array_equal(pr[k], full[k]), k
