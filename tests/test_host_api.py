"""Host-side mirror of the JaxDEM API: registry, State/System construction, and the
unsupported-configuration errors (all raised before any device call)."""

from __future__ import annotations

import warnings

import numpy as np
import pytest

import jaxdem_gb300 as jdem
from jaxdem_gb300.factory import _normalize_key

F32 = np.float32


def test_key_normalization():
    """factory.py:28-35 / tests/test_public_api.py:24-36."""
    for k in ("CellList", "cell_list", "cell-list", "Cell List", "celllist"):
        assert _normalize_key(k) == "celllist"
        assert type(jdem.Collider.create(k, state=jdem.State.create(pos=np.zeros((2, 3))))).__name__ == "DynamicCellList"


def test_unknown_key_and_unknown_kwargs():
    with pytest.raises(KeyError):
        jdem.Collider.create("no_such_collider")
    st = jdem.State.create(pos=np.zeros((2, 3)))
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        jdem.Collider.create("CellList", state=st, bogus=3)  # factory.py:479-492: dropped, warned
        assert any("ignoring unknown keyword" in str(x.message) for x in w)
    with pytest.raises(TypeError):  # Domain.Create forwards **kw to the constructor
        jdem.Domain.create("periodic", dim=2, box_size=[1.0, 1.0], bogus=3)


def test_duplicate_registration_rejected():
    class Other(jdem.Collider):
        pass

    with pytest.raises(ValueError):
        jdem.Collider.register("CellList")(Other)


def test_state_create_defaults():
    """state.py:640-862: mass from the material table, inertia 0.4 m r^2, relabelled clumps."""
    mats = [jdem.Material.create("elastic", young=1e3, poisson=0.3, density=2.0)]
    table = jdem.MaterialTable.from_materials(mats)
    st = jdem.State.create(pos=np.zeros((3, 3)), rad=[0.5, 1.0, 0.5], mat_table=table)
    vol = 4.0 / 3.0 * np.pi * np.array([0.125, 1.0, 0.125])
    assert np.allclose(st.mass, 2.0 * vol, rtol=1e-6)
    assert np.allclose(st.inertia[:, 0], 0.4 * st.mass * st.rad ** 2, rtol=1e-6)
    assert st.q.w.shape == (3, 1) and np.all(st.q.w == 1)
    assert np.array_equal(st.clump_id, [0, 1, 2])
    st2 = jdem.State.create(pos=np.zeros((3, 2)), clump_id=[7, 7, 3])
    assert np.array_equal(st2.clump_id, [1, 1, 0])
    assert st2.ang_vel.shape == (3, 1)


def test_bond_table_is_symmetrised():
    """state.py:735-761: bonds given one way become symmetric, -1 padded."""
    st = jdem.State.create(pos=np.zeros((3, 2)), bond_id=[[1], [2], [-1]])
    rows = [set(r[r >= 0].tolist()) for r in st.bond_id]
    assert rows == [{1}, {0, 2}, {1}]


def test_harmonic_and_linear_matchers():
    mats = [jdem.Material.create("elastic", young=1e3, poisson=0.3),
            jdem.Material.create("elastic", young=3e3, poisson=0.3)]
    h = jdem.MaterialTable.from_materials(mats)
    lin = jdem.MaterialTable.from_materials(mats, matcher=jdem.MaterialMatchmaker.create("linear"))
    assert np.isclose(h.young_eff[0, 1], 2 * 1e3 * 3e3 / 4e3)
    assert np.isclose(lin.young_eff[0, 1], 2e3)


def test_system_create_components_and_validation():
    st = jdem.State.create(pos=np.random.default_rng(0).uniform(0, 5, (20, 3)), rad=np.full(20, 0.5))
    sy = jdem.System.create(state=st, collider_type="CellList", domain_type="periodic",
                            domain_kw=dict(box_size=[5, 5, 5]), dt=1e-3)
    assert sy.collider.type_name == "celllist" and np.isclose(sy.collider.cell_size, 1.0)
    assert sy.collider.neighbor_mask.shape == (27, 3)
    assert sy.domain.periodic and np.allclose(sy.domain.inv_box_size, 0.2)
    with pytest.raises(ValueError):
        jdem.System.create(state_shape=(4, 3), state=st)
    with pytest.raises(TypeError):
        jdem.System.create()
    with pytest.raises(ValueError):
        jdem.System.create(state=st, domain_type="periodic", domain_kw=dict(box_size=[5, 5]))
    with pytest.raises(ValueError):
        jdem.System.create(state=st, domain_type="reflect", domain_kw=dict(box_size=[5, 5, 5],
                                                                            restitution_coefficient=1.5))


def test_unsupported_configurations_raise_before_device_work():
    from jaxdem_gb300 import session

    st2 = jdem.State.create(pos=np.zeros((4, 3)))
    fm = jdem.ForceManager.create((4, 3), force_functions=[lambda p, s, y: (p, p)])
    sy2 = jdem.System.create(state=st2, collider_type="CellList", force_manager=fm)
    with pytest.raises(NotImplementedError):
        session.engine_for(st2, sy2)
    sy3 = jdem.System.create(state=st2, collider_type="CellList",
                             user_pre_step_actions=lambda s, y: (s, y))
    with pytest.raises(NotImplementedError):
        session.engine_for(st2, sy3)


def test_trajectory_rollout_argument_checks():
    st = jdem.State.create(pos=np.zeros((2, 3)))
    sy = jdem.System.create(state=st)
    with pytest.raises(ValueError):
        jdem.System.trajectory_rollout(st, sy)
    with pytest.raises(ValueError):
        jdem.System.trajectory_rollout(st, sy, strides=np.ones((2, 2), int))


def test_hertz_force_model_pair_constant():
    """HertzianForce (forces/hertz.py:22-170) reads young and poisson per material; the
    engine receives (4/3) E* per material pair in the reference's float32 order."""
    from jaxdem_gb300 import session
    from oracle import dem_ref as R

    mats = [jdem.Material.create("elastic", young=1e3, poisson=0.3),
            jdem.Material.create("elastic", young=4e3, poisson=0.2)]
    table = jdem.MaterialTable.from_materials(mats)
    st = jdem.State.create(pos=np.zeros((2, 3)), mat_table=table)
    sy = jdem.System.create(state=st, mat_table=table, force_model_type="hertz")
    assert type(sy.force_model).__name__ == "HertzianForce"
    law, k, props = session.pair_law(sy)
    assert law == "hertz" and k.dtype == F32 and props is None
    assert np.array_equal(k, R.hertz_constant([1e3, 4e3], [0.3, 0.2]))
    e_star = 1.0 / ((1 - 0.09) / 1e3 + (1 - 0.04) / 4e3)
    assert np.isclose(k[0, 1], 4.0 / 3.0 * e_star, rtol=1e-6) and k[0, 1] == k[1, 0]
    law, k, _ = session.pair_law(jdem.System.create(state=st, mat_table=table))
    assert law == "spring" and np.array_equal(k, table.young_eff)


def test_cundall_strack_material_tables():
    """CundallStrackForce (forces/cundall_strack.py:22-242) reads young, poisson, e, mu and
    mu_r per material (elasticfrict, materials/elastic_mats.py:29-47); the engine gets the
    damping ratio per material pair and (young, G, mu, mu_r) per material, equal to the
    oracle's independent restatement bit for bit."""
    from jaxdem_gb300 import session
    from oracle import dem_ref as R

    mats = [jdem.Material.create("elasticfrict", young=1e3, poisson=0.25, e=0.6, mu=0.4, mu_r=0.05),
            jdem.Material.create("elasticfrict", young=3e3, poisson=0.3, e=0.0, mu=0.3)]
    table = jdem.MaterialTable.from_materials(mats)
    st = jdem.State.create(pos=np.zeros((2, 3)), mat_table=table, mat_id=[0, 1])
    sy = jdem.System.create(state=st, mat_table=table, force_model_type="cundallstrack")
    assert type(sy.force_model).__name__ == "CundallStrackForce"
    law, beta, props = session.pair_law(sy)
    rb, rp = R.cs_tables([1e3, 3e3], [0.25, 0.3], [0.6, 0.0], [0.4, 0.3], [0.05, 0.0])
    assert law == "cundallstrack" and np.array_equal(beta, rb) and np.array_equal(props, rp)
    # e = 0 takes the analytic limit beta = 1 (no NaN); G = E / (2 (1 + nu))
    assert beta[1, 1] == 1.0 and beta[0, 1] == 1.0 and np.isfinite(beta).all()
    assert np.isclose(props[0, 1], 1e3 / 2.5) and np.isclose(beta[0, 0], -np.log(0.6) / np.sqrt(np.pi ** 2 + np.log(0.6) ** 2))


def test_rollout_frame_times_match_stepwise_float32():
    """Frame times of a rollout: float32 ``time += dt`` once per step (system.py:62-66),
    for a scalar system and for a batch with per-member dt and time."""
    from jaxdem_gb300 import session

    strides = np.array([0, 3, 7, 0, 5, 1], np.int64)
    st = jdem.State.create(pos=np.zeros((2, 3)))
    sy = jdem.System.create(state=st, dt=1e-3, time=0.1)
    times, counts = session._frame_times(sy, strides, batched=False)
    t, ref = F32(0.1), []
    for k in strides:
        for _ in range(k):
            t = F32(t + F32(1e-3))
        ref.append(t)
    assert times.dtype == F32 and np.array_equal(times, ref)
    assert np.array_equal(counts, np.cumsum(strides))
    bsy = jdem.System.stack([jdem.System.create(state=st, dt=dt, time=t0) for dt, t0 in ((1e-3, 0.0), (3e-4, 2.0))])
    times, counts = session._frame_times(bsy, strides, batched=True)
    assert times.shape == (len(strides), 2) and counts.shape == (len(strides), 2)
    for b, (dt, t0) in enumerate(((1e-3, 0.0), (3e-4, 2.0))):
        t, ref = F32(t0), []
        for k in strides:
            for _ in range(k):
                t = F32(t + F32(dt))
            ref.append(t)
        assert np.array_equal(times[:, b], ref)


def test_empty_rollout_frames_have_a_zero_frame_axis():
    from jaxdem_gb300 import session

    st = jdem.State.create(pos=np.zeros((4, 2)))
    sy = jdem.System.create(state=st)
    stacked = session._stack_frames([(st, sy)])
    es, ey = session._empty_frames(stacked)
    assert es.pos_c.shape == (0, 4, 2) and es.q.w.shape == (0, 4, 1)
    assert np.shape(ey.time) == (0,) and ey.domain.box_size.shape[0] == 0


def test_grid_state_lattice():
    st = jdem.utils.grid_state(n_per_axis=(2, 3), spacing=1.5, radius=0.4, seed=1)
    assert st.pos_c.shape == (6, 2)
    assert np.allclose(sorted(set(st.pos_c[:, 1].tolist())), [0.0, 1.5, 3.0])
    assert np.all((st.vel >= -1) & (st.vel <= 1))


def test_neighbor_list_collider_create():
    """NeighborList.Create (colliders/neighbor_list.py:287-440): absolute skin or a
    fraction of the cutoff (default 0.05), not both; the estimated max_neighbors; a
    cutoff below the largest contact distance is refused (the device list never drops
    contacts, the reference would)."""
    import jaxdem_gb300 as jdem

    rng = np.random.default_rng(0)
    st = jdem.State.create(pos=rng.uniform(0, 10, (200, 3)), rad=np.full(200, 0.5))
    c = jdem.Collider.create("NeighborList", state=st, cutoff=1.0, skin=0.2)
    assert type(c).__name__ == "NeighborList" and c.type_name == "neighborlist"
    assert np.isclose(c.skin, 0.2) and np.isclose(c.cutoff, 1.0) and c.max_neighbors >= 1
    assert np.isclose(jdem.Collider.create("NeighborList", state=st, cutoff=1.2).skin, 0.06)
    assert np.isclose(jdem.Collider.create("NeighborList", state=st, cutoff=1.0, skin_fraction=0.5).skin, 0.5)
    with pytest.raises(ValueError):
        jdem.Collider.create("NeighborList", state=st, cutoff=1.0, skin=0.1, skin_fraction=0.1)
    with pytest.raises(NotImplementedError):
        jdem.Collider.create("NeighborList", state=st, cutoff=0.8)
    assert jdem.Collider.create("NeighborList", state=st, cutoff=1.0, max_neighbors=17).max_neighbors == 17
