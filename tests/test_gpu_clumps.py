"""Rigid clumps (State.add_clump, state.py:1230-1420) on the device, through the C ABI,
against the oracle's restatement.

Each clump's state is held once on the device and its members' world positions
pos_c + R(q) pos_p feed the cell list; contact forces and their lever-arm
torques are summed per clump (ForceManager.apply, force_manager.py:338-425) and
the integrators advance the clump.  The oracle is pinned by closed forms in
test_oracle_pins.py and by the reference's own outputs for clumps (spring and
Cundall-Strack contacts, periodic and reflect boxes, create_neighbor_list) in
tests/golden.  Bars: per-sphere force and torque <= 1e-5 floored relative error
from identical inputs; rollouts <= 1e-4 in position; energies; bit-exact
contact sets and neighbour lists without same-clump pairs.
"""

from __future__ import annotations

import numpy as np
import pytest

import jaxdem_gb300 as jdem
from jaxdem_gb300._lib import Engine, JdemError
from oracle import dem_ref as R
from tests.helpers import force_err, min_image_diff

pytestmark = pytest.mark.gpu

F32 = np.float32
K = np.array([[1e3]], F32)


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def random_quats(rng, n, dim):
    if dim == 2:
        a = rng.uniform(0, 2 * np.pi, n)
        return np.stack([np.cos(a / 2), 0 * a, 0 * a, np.sin(a / 2)], 1)
    q = rng.normal(size=(n, 4))
    return q / np.linalg.norm(q, axis=1, keepdims=True)


def clump_system(n_clumps=500, dim=3, seed=61, phi=0.35, spin=1.0):
    """Dumbbells and triangles of spheres (radius 0.4-0.5) at random centres and
    orientations in a periodic box; per-member arrays in the reference layout."""
    rng = np.random.default_rng(seed)
    sizes = rng.choice([1, 2, 3], n_clumps, p=[0.2, 0.5, 0.3])
    N = int(sizes.sum())
    rad = rng.uniform(0.4, 0.5, N).astype(F32)
    vol = (4 / 3 * np.pi * rad ** 3) if dim == 3 else (np.pi * rad ** 2)
    L = float((vol.sum() / phi) ** (1 / dim))
    cid = np.repeat(np.arange(n_clumps), sizes)
    pp = np.zeros((N, dim))
    k = 0
    for s in sizes:
        offs = {1: [[0.0] * dim], 2: [[-0.35] + [0.0] * (dim - 1), [0.35] + [0.0] * (dim - 1)],
                3: [[-0.3, -0.2] + [0.0] * (dim - 2), [0.3, -0.2] + [0.0] * (dim - 2), [0.0, 0.35] + [0.0] * (dim - 2)]}[s]
        pp[k:k + s] = offs
        k += s
    centres = rng.uniform(0, L, (n_clumps, dim))
    qc = random_quats(rng, n_clumps, dim)
    vc = rng.normal(0, 0.3, (n_clumps, dim))
    ad = 3 if dim == 3 else 1
    wc = rng.normal(0, spin, (n_clumps, ad))
    Mc = np.bincount(cid, weights=vol)  # density 1
    Ic = np.stack([Mc * 0.2 + 0.05 * a for a in range(ad)], 1)
    return dict(dim=dim, L=L, N=N, rad=rad, clump_id=cid.astype(np.int32), pos_p=pp.astype(F32),
                pos_c=centres[cid].astype(F32), q=qc[cid].astype(F32), vel=vc[cid].astype(F32),
                ang_vel=wc[cid].astype(F32), mass=Mc[cid].astype(F32), inertia=Ic[cid].astype(F32))


def engine(c, domain="periodic", linear="verlet", rotation="verletspiral", skin=0.1, gravity=None):
    d = c["dim"]
    desc = dict(n=c["N"], domain=domain, linear=linear, rotation=rotation, dt=1e-3, box_size=np.full(d, c["L"], F32),
                anchor=np.zeros(d, F32), restitution=1.0, gravity=np.zeros(d, F32) if gravity is None else gravity,
                cell_size=1.0, search_range=1)
    return Engine(d, [desc], K, skin=skin)


def upload(eng, c, **extra):
    eng.upload(pos=c["pos_c"], rad=c["rad"], mass=c["mass"], vel=c["vel"], q=c["q"], ang_vel=c["ang_vel"],
               inertia=c["inertia"], pos_p=c["pos_p"], clump_id=c["clump_id"], **extra)


def ostate_sys(c, domain="periodic", linear="verlet", rotation="verletspiral", gravity=None):
    d = c["dim"]
    st = R.make_state(c["pos_c"], vel=c["vel"], rad=c["rad"], mass=c["mass"], q=c["q"], ang_vel=c["ang_vel"],
                      inertia=c["inertia"], pos_p=c["pos_p"], clump_id=c["clump_id"])
    cell, mask = R.cell_list_create(c["rad"], d)
    sy = R.OSystem(dim=d, domain=domain, box_size=np.full(d, c["L"], F32), anchor=np.zeros(d, F32),
                   young_eff=K, dt=F32(1e-3), cell_size=cell, neighbor_mask=mask,
                   gravity=np.zeros(d, F32) if gravity is None else np.asarray(gravity, F32), linear=linear,
                   rotation=rotation)
    return st, sy


@pytest.mark.parametrize("dim", [3, 2])
def test_clump_force_and_torque_per_sphere(dim):
    c = clump_system(dim=dim, seed=61 + dim)
    st, sy = ostate_sys(c)
    f64, t64 = R.cell_list_force(st, sy, sum_dtype=np.float64)
    eng = engine(c)
    try:
        upload(eng, c)
        eng.compute_force()
        out = eng.download()
        pairs = eng.contacts()
        e = eng.energy()
    finally:
        eng.close()
    assert np.abs(t64).max() > 0
    assert force_err(out["force"], f64) <= 1e-5
    assert force_err(out["torque"], t64) <= 1e-5
    # members report their clump's centre, orientation and spin
    assert np.array_equal(out["pos_c"], c["pos_c"]) and np.array_equal(out["ang_vel"], c["ang_vel"])
    assert np.array_equal(pairs, R.contact_pairs(st, sy))
    assert not np.any(c["clump_id"][pairs[:, 0]] == c["clump_id"][pairs[:, 1]])
    ref = R.compute_energy(st, sy)
    for k in range(4):
        assert abs(e[k] - ref[k]) <= 1e-5 * max(abs(ref[k]), 1e-3 * abs(ref[2]))


@pytest.mark.parametrize("dim,domain,linear,gravity", [(3, "periodic", "verlet", None), (2, "periodic", "verlet", None),
                                                       (3, "free", "verlet", [0.0, -1.0, 0.0]),
                                                       (3, "periodic", "euler", None)])
def test_clump_rollout_matches_oracle(dim, domain, linear, gravity, steps=50):
    c = clump_system(n_clumps=400, dim=dim, seed=70 + dim)
    g = None if gravity is None else np.asarray(gravity, F32)
    st, sy = ostate_sys(c, domain=domain, linear=linear, gravity=g)
    st, sy = R.step(st, sy, steps, sum_dtype=np.float64)
    eng = engine(c, domain=domain, linear=linear, gravity=g)
    try:
        upload(eng, c)
        eng.step(steps)
        out = eng.download()
        box, anc = eng.domain_state()
    finally:
        eng.close()
    per = np.full(dim, c["L"]) if domain == "periodic" else None
    assert min_image_diff(out["pos_c"], st.pos_c, per) <= 1e-4
    assert np.abs(out["vel"] - st.vel).max() <= 1e-3 * max(1.0, np.abs(st.vel).max())
    assert np.abs(out["ang_vel"] - st.ang_vel).max() <= 1e-3 * max(1.0, np.abs(st.ang_vel).max())
    assert np.abs(out["q"] - st.q).max() <= 1e-4
    assert force_err(out["force"], st.force) <= 1e-3
    # every member reports its clump's state
    for k in ("pos_c", "vel", "q", "ang_vel", "force", "torque"):
        first = np.zeros(int(c["clump_id"].max()) + 1, int)
        first[c["clump_id"][::-1]] = np.arange(c["N"])[::-1]
        assert np.array_equal(out[k], out[k][first[c["clump_id"]]]), k
    if domain == "free":
        assert np.allclose(box[0], sy.box_size, rtol=1e-5, atol=1e-5)
        assert np.allclose(anc[0], sy.anchor, rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("dim", [3, 2])
def test_clump_reflect_rollout_matches_oracle(dim, steps=200):
    """Clumps falling onto the floor of a reflect box (reflect.py:165-297): wall impulses
    with spin, the clump's collision fraction and the remaining-step corrections."""
    c = clump_system(n_clumps=300, dim=dim, seed=85 + dim, phi=0.25)
    # every member inside the box at the start (|pos_p| + rad <= 0.85)
    c["pos_c"] = (1.0 + c["pos_c"] * (c["L"] - 2.0) / c["L"]).astype(F32)
    g = np.zeros(dim, F32)
    g[1] = -20.0
    st, sy = ostate_sys(c, domain="reflect", gravity=g)
    sy.restitution = F32(0.7)
    st, sy = R.step(st, sy, steps, sum_dtype=np.float64)
    desc = dict(n=c["N"], domain="reflect", linear="verlet", rotation="verletspiral", dt=1e-3,
                box_size=np.full(dim, c["L"], F32), anchor=np.zeros(dim, F32), restitution=0.7, gravity=g,
                cell_size=1.0, search_range=1)
    eng = Engine(dim, [desc], K, skin=0.1)
    try:
        upload(eng, c)
        eng.step(steps)
        out = eng.download()
    finally:
        eng.close()
    assert min_image_diff(out["pos_c"], st.pos_c) <= 1e-4
    assert np.abs(out["vel"] - st.vel).max() <= 1e-3 * max(1.0, np.abs(st.vel).max())
    assert np.abs(out["ang_vel"] - st.ang_vel).max() <= 1e-3 * max(1.0, np.abs(st.ang_vel).max())
    assert np.abs(out["q"] - st.q).max() <= 1e-4
    # clumps hit the floor and bounced
    assert np.any(st.vel[:, 1] > 0.5)


CS_MATS = dict(young=[1e3, 3e3], poisson=[0.25, 0.3], e=[0.6, 0.8], mu=[0.4, 0.3], mu_r=[0.05, 0.1])


def cs_engine_sys(c, domain="periodic", gravity=None, rotation="verletspiral"):
    """Clumps with Cundall-Strack contacts: two materials drawn per sphere."""
    d = c["dim"]
    beta, props = R.cs_tables(**CS_MATS)
    c = dict(c, mat_id=np.random.default_rng(c["N"]).integers(0, 2, c["N"]).astype(np.int32))
    g = np.zeros(d, F32) if gravity is None else np.asarray(gravity, F32)
    desc = dict(n=c["N"], domain=domain, linear="verlet", rotation=rotation, dt=5e-4, box_size=np.full(d, c["L"], F32),
                anchor=np.zeros(d, F32), restitution=1.0, gravity=g, cell_size=1.0, search_range=1)
    eng = Engine(d, [desc], beta, skin=0.1, force_law="cundallstrack", material_props=props)
    st, sy = ostate_sys(c, domain=domain, rotation=rotation, gravity=g)
    st.mat_id = c["mat_id"]
    sy.young_eff, sy.mat_props, sy.force_law, sy.dt = beta, props, "cundallstrack", F32(5e-4)
    return c, eng, st, sy


@pytest.mark.parametrize("dim", [3, 2])
def test_clumps_with_cundall_strack_match_oracle(dim, steps=40):
    """Cundall-Strack contacts between clumps (cundall_strack.py:100-196 on the members'
    world positions with their clump's velocity, spin and mass; the lever torque
    cross(R(q) pos_p, F) added, cell_list.py:452-464; clump sums, force_manager.py:338-425)."""
    c = clump_system(n_clumps=400, dim=dim, seed=110 + dim, spin=2.0)
    c, eng, st, sy = cs_engine_sys(c)
    f64, t64 = R.cell_list_force(st, sy, sum_dtype=np.float64)
    e_ref = R.compute_energy(st, sy)
    st2, _ = R.step(st.copy(), sy, steps, sum_dtype=np.float64)
    try:
        upload(eng, c, mat_id=c["mat_id"])
        eng.compute_force()
        f0 = eng.download()
        e = eng.energy()
        upload(eng, c, mat_id=c["mat_id"])
        eng.step(steps)
        out = eng.download()
    finally:
        eng.close()
    assert np.abs(t64).max() > 0
    assert force_err(f0["force"], f64) <= 1e-5
    assert force_err(f0["torque"], t64) <= 1e-5
    for k in range(4):
        assert abs(e[k] - e_ref[k]) <= 1e-5 * max(abs(e_ref[k]), 1e-3 * abs(e_ref[2]))
    assert min_image_diff(out["pos_c"], st2.pos_c, np.full(dim, c["L"])) <= 1e-4
    assert np.abs(out["vel"] - st2.vel).max() <= 1e-3 * max(1.0, np.abs(st2.vel).max())
    assert np.abs(out["ang_vel"] - st2.ang_vel).max() <= 1e-3 * max(1.0, np.abs(st2.ang_vel).max())
    assert np.abs(out["q"] - st2.q).max() <= 1e-4


def test_clumps_with_cundall_strack_in_a_reflect_box(steps=100):
    """2D clumps under gravity with the spiral integrator, wall impulses and friction."""
    c = clump_system(n_clumps=300, dim=2, seed=121, phi=0.25, spin=2.0)
    c["pos_c"] = (1.0 + c["pos_c"] * (c["L"] - 2.0) / c["L"]).astype(F32)
    c, eng, st, sy = cs_engine_sys(c, domain="reflect", gravity=[0.0, -10.0], rotation="spiral")
    st2, _ = R.step(st.copy(), sy, steps, sum_dtype=np.float64)
    try:
        upload(eng, c, mat_id=c["mat_id"])
        eng.step(steps)
        out = eng.download()
    finally:
        eng.close()
    assert min_image_diff(out["pos_c"], st2.pos_c) <= 1e-4
    assert np.abs(out["vel"] - st2.vel).max() <= 1e-3 * max(1.0, np.abs(st2.vel).max())
    assert np.abs(out["ang_vel"] - st2.ang_vel).max() <= 1e-3 * max(1.0, np.abs(st2.ang_vel).max())


@pytest.mark.parametrize("dim", [3, 2])
def test_clump_neighbor_list_matches_oracle(dim):
    """create_neighbor_list on a clump handle (cell_list.py:498-595): the members' world
    positions, no member listing another member of its clump, bit for bit."""
    c = clump_system(n_clumps=500, dim=dim, seed=130 + dim)
    st, sy = ostate_sys(c)
    cutoff = 2.5 * float(c["rad"].max())
    want, want_ovf = R.create_neighbor_list(st, sy, cutoff, 40)
    eng = engine(c)
    try:
        upload(eng, c)
        nl, ovf = eng.neighbor_list(cutoff, 40)
    finally:
        eng.close()
    assert bool(ovf) == bool(want_ovf)
    assert np.array_equal(nl, want)
    rows = np.repeat(np.arange(c["N"]), 40).reshape(c["N"], 40)
    ok = nl >= 0
    assert ok.sum() > 0 and not np.any(c["clump_id"][rows[ok]] == c["clump_id"][nl[ok]])


def test_clumps_through_the_public_api():
    """State.add_clump builds the bodies; System.step and trajectory_rollout run them."""
    rng = np.random.default_rng(90)
    st = jdem.State.create(pos=np.zeros((0, 3)))
    L = 9.0
    for k in range(60):
        centre = rng.uniform(0, L, 3)
        pts = centre + np.array([[-0.35, 0, 0], [0.35, 0, 0]])
        st = jdem.State.add_clump(st, pts, rad=[0.45, 0.45], mass=1.0, inertia=[0.2, 0.3, 0.3],
                                  vel=rng.normal(0, 0.5, 3), ang_vel=rng.normal(0, 1.0, 3))
    sy = jdem.System.create(state=st, collider_type="CellList", domain_type="periodic", dt=1e-3,
                            domain_kw=dict(box_size=[L] * 3, anchor=[0.0] * 3))
    st2, _ = jdem.System.step(st, sy, n=20)
    ost = R.make_state(st.pos_c, vel=st.vel, rad=st.rad, mass=st.mass, q=st.q.as_array(), ang_vel=st.ang_vel,
                       inertia=st.inertia, pos_p=st.pos_p, clump_id=st.clump_id)
    cell, mask = R.cell_list_create(st.rad, 3)
    osy = R.OSystem(dim=3, domain="periodic", box_size=np.full(3, L, F32), anchor=np.zeros(3, F32),
                    young_eff=np.asarray(sy.mat_table.young_eff, F32), dt=F32(1e-3), cell_size=cell,
                    neighbor_mask=mask, gravity=np.zeros(3, F32))
    ost, _ = R.step(ost, osy, 20, sum_dtype=np.float64)
    assert min_image_diff(st2.pos_c, ost.pos_c, np.full(3, L)) <= 1e-5
    assert np.abs(st2.ang_vel - ost.ang_vel).max() <= 1e-4
    _, _, (frames, _) = jdem.System.trajectory_rollout(st, sy, n=4, stride=5)
    assert np.array_equal(frames.pos_c[-1], st2.pos_c) and np.array_equal(frames.q.w[-1], st2.q.w)
