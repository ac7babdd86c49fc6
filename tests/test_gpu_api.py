"""The reference-facing API (State / System / Factory types) running on the GPU engine."""

from __future__ import annotations

import numpy as np
import pytest

import jaxdem_gb300 as jdem
from jaxdem_gb300 import workloads as W
from jaxdem_gb300.batch import step_many
from oracle import dem_ref as R
from tests.helpers import force_err, min_image_diff

pytestmark = pytest.mark.gpu

F32 = np.float32


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def make(N=1024, seed=3, phi=0.45, dim=3, domain="periodic", gravity=None):
    rng = np.random.Generator(np.random.PCG64(seed))
    w = W.periodic_system("t", rng, N, dim, rng.choice([0.5, 0.6], size=N), phi, 0.1, 1e-3, 10)
    mats = [jdem.Material.create("elastic", young=1e3, poisson=0.3, density=1.0)]
    table = jdem.MaterialTable.from_materials(mats)
    st = jdem.State.create(pos=w.pos, vel=w.vel, rad=w.rad, mat_table=table)
    sy = jdem.System.create(state=st, collider_type="CellList", domain_type=domain, mat_table=table, dt=1e-3,
                            domain_kw=dict(box_size=w.box_size, anchor=w.anchor),
                            force_manager_kw=None if gravity is None else {"gravity": gravity})
    return w, st, sy


def test_system_step_matches_oracle_and_advances_time():
    w, st, sy = make()
    st2, sy2 = jdem.System.step(st, sy, n=20)
    ost = R.make_state(w.pos, vel=w.vel, rad=w.rad, mass=st.mass)
    cell, mask = R.cell_list_create(w.rad, 3)
    osy = R.OSystem(dim=3, domain="periodic", box_size=w.box_size, anchor=w.anchor, young_eff=np.array([[1e3]], F32),
                    dt=F32(1e-3), cell_size=cell, neighbor_mask=mask, gravity=np.zeros(3, F32))
    ost, osy = R.step(ost, osy, 20, sum_dtype=np.float64)
    assert min_image_diff(st2.pos_c, ost.pos_c, w.box_size) <= 1e-5
    assert force_err(st2.force, ost.force) <= 1e-4
    assert int(sy2.step_count) == 20
    assert np.isclose(float(sy2.time), float(osy.time))


def test_trajectory_rollout_frames():
    """system.py:606-699: frames saved after their steps; a leading stride of 0 records the
    initial state (tests/test_public_api.py:69-78)."""
    w, st, sy = make(N=512)
    fs, fy, traj = jdem.System.trajectory_rollout(st, sy, strides=np.array([0, 5, 5]))
    states, systems = traj
    assert states.pos_c.shape == (3, 512, 3)
    assert np.array_equal(states.pos_c[0], st.pos_c)
    assert np.array_equal(systems.step_count, [0, 5, 10])
    ref, _ = jdem.System.step(st, sy, n=10)
    assert np.array_equal(fs.pos_c, states.pos_c[-1])
    assert min_image_diff(fs.pos_c, ref.pos_c, w.box_size) <= 1e-6
    fs2, _, traj2 = jdem.System.trajectory_rollout(st, sy, n=4, stride=3, save_fn=lambda s, y: s.vel)
    assert traj2.shape == (4, 512, 3)


def test_vmapped_batch_matches_members():
    """A leading batch axis steps B independent systems (system.py:743-744)."""
    members = [make(N=700, seed=s) for s in (1, 2, 3)]
    # equal N, equal box for a stacked batch
    box = members[0][0].box_size
    sts = []
    for w, st, sy in members:
        st.pos_c = np.mod(st.pos_c, box).astype(F32)
        sts.append(st)
    bst = jdem.State.stack(sts)
    bsy = members[0][2]
    out, _ = jdem.System.step(bst, bsy, n=15)
    for b, st in enumerate(sts):
        alone, _ = jdem.System.step(st, bsy, n=15)
        assert min_image_diff(out.pos_c[b], alone.pos_c, box) <= 1e-5


def test_step_many_uneven_systems():
    items = [make(N=n, seed=s, phi=p) for n, s, p in ((128, 5, 0.3), (2000, 6, 0.5), (640, 7, 0.55))]
    items.append(make(N=900, seed=8, dim=2, phi=0.6, domain="reflect", gravity=[0.0, -1.0]))
    sts, sys_ = step_many([i[1] for i in items], [i[2] for i in items], 25)
    for (w, st, sy), st2, sy2 in zip(items, sts, sys_):
        alone, _ = jdem.System.step(st, sy, n=25)
        box = w.box_size if w.domain == "periodic" else None
        assert min_image_diff(st2.pos_c, alone.pos_c, box) <= 1e-5
        assert int(sy2.step_count) == 25
    # a second call on batches of the same shape reuses the cached handle: same results,
    # no new handle (the input states are not modified by the first call)
    from jaxdem_gb300 import session

    n_handles = len(session._CACHE)
    again, _ = step_many([i[1] for i in items], [i[2] for i in items], 25)
    assert len(session._CACHE) == n_handles
    for a, b in zip(sts, again):
        assert np.array_equal(a.pos_c, b.pos_c) and np.array_equal(a.vel, b.vel)


def test_collider_slot_and_pair_forces():
    w, st, sy = make(N=800, phi=0.55)
    st_f, _ = sy.collider.compute_force(st, sy)
    ost = R.make_state(w.pos, rad=w.rad)
    cell, mask = R.cell_list_create(w.rad, 3)
    osy = R.OSystem(dim=3, domain="periodic", box_size=w.box_size, anchor=w.anchor, young_eff=np.array([[1e3]], F32),
                    dt=F32(1e-3), cell_size=cell, neighbor_mask=mask, gravity=np.zeros(3, F32))
    ref, _ = R.cell_list_force(ost, osy, sum_dtype=np.float64)
    assert force_err(st_f.force, ref) <= 1e-5
    _, _, pe = sy.collider.compute_potential_energy(st, sy)
    assert np.isclose(pe, R.cell_list_energy(ost, osy, sum_dtype=np.float64), rtol=1e-5)
    _, _, ids, f = jdem.utils.get_pair_forces_and_ids(st, sy)
    hit = np.linalg.norm(f, axis=1) > 0
    got = {tuple(sorted(p)) for p in ids[hit].tolist()}
    want = {tuple(p) for p in R.contact_pairs(ost, osy).tolist()}
    assert got == want
    assert np.array_equal(jdem.utils.contact_pairs(st, sy), R.contact_pairs(ost, osy))


def test_neighbor_list_collider_steps_like_cell_list():
    """The NeighborList collider type (colliders/neighbor_list.py) runs the same device
    path with its own skin and initial capacity: same trajectory as CellList."""
    w, st, sy = make(N=1500, seed=11, phi=0.5)
    mats = [jdem.Material.create("elastic", young=1e3, poisson=0.3, density=1.0)]
    table = jdem.MaterialTable.from_materials(mats)
    sy_nl = jdem.System.create(state=st, collider_type="NeighborList", collider_kw=dict(cutoff=1.2, skin=0.2),
                               domain_type="periodic", mat_table=table, dt=1e-3,
                               domain_kw=dict(box_size=w.box_size, anchor=w.anchor))
    a, _ = jdem.System.step(st, sy, n=40)
    b, sy_b = jdem.System.step(st, sy_nl, n=40)
    assert min_image_diff(b.pos_c, a.pos_c, w.box_size) <= 1e-5
    assert force_err(b.force, a.force) <= 1e-4
    assert int(sy_b.step_count) == 40
    _, _, pe = sy_nl.collider.compute_potential_energy(b, sy_b)
    _, _, pe_ref = sy.collider.compute_potential_energy(b, sy)
    assert np.isclose(pe, pe_ref, rtol=1e-5)
