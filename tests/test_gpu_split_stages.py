"""System.step replayed stage by stage through the split factory types.

``_step_once`` (system.py:60-82) calls, in order, ``domain.apply``, the linear
and rotation integrators' ``step_before_force``, ``collider.compute_force``,
``force_manager.apply`` and the integrators' ``step_after_force``.  Each of
those methods of the host types runs its stage on the GPU (jdem_domain_apply,
jdem_integrate, jdem_compute_force, jdem_force_manager_apply), so code that
drives the stages itself gets the fused ``System.step``'s result: positions,
velocities and forces bit for bit over several steps, in a periodic box, a
reflecting box with gravity and a free domain (whose box follows the spheres).
"""

from __future__ import annotations

import dataclasses

import numpy as np
import pytest

import jaxdem_gb300 as jdem
from jaxdem_gb300 import workloads as W

pytestmark = pytest.mark.gpu

F32 = np.float32


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def make(domain, dim, N=2048, seed=5, gravity=None, rotation="verletspiral"):
    rng = np.random.Generator(np.random.PCG64(seed))
    w = W.periodic_system("t", rng, N, dim, rng.choice([0.5, 0.6], size=N), 0.45, 0.1, 1e-3, 10)
    mats = [jdem.Material.create("elastic", young=1e3, poisson=0.3, density=1.0)]
    table = jdem.MaterialTable.from_materials(mats)
    pos = w.pos
    if domain == "reflect":  # spheres inside the walls
        pos = np.clip(pos, w.rad[:, None] + 0.01, np.asarray(w.box_size, F32) - w.rad[:, None] - 0.01).astype(F32)
    st = jdem.State.create(pos=pos, vel=w.vel, rad=w.rad, mat_table=table)
    sy = jdem.System.create(state=st, collider_type="CellList", domain_type=domain, mat_table=table, dt=1e-3,
                            rotation_integrator_type=rotation,
                            domain_kw=dict(box_size=w.box_size, anchor=w.anchor),
                            force_manager_kw=None if gravity is None else {"gravity": gravity})
    return st, sy


def step_by_stages(state, system):
    """_step_once (system.py:60-82) through the types' own stage methods."""
    system = dataclasses.replace(system, time=F32(system.time + system.dt), step_count=system.step_count + 1)
    state, system = system.domain.apply(state, system)
    system = dataclasses.replace(system, domain=dataclasses.replace(
        system.domain, inv_box_size=(F32(1.0) / system.domain.box_size).astype(F32)))
    state, system = system.linear_integrator.step_before_force(state, system)
    state, system = system.rotation_integrator.step_before_force(state, system)
    state, system = system.collider.compute_force(state, system)
    state, system = system.force_manager.apply(state, system)
    state, system = system.linear_integrator.step_after_force(state, system)
    state, system = system.rotation_integrator.step_after_force(state, system)
    return state, system


@pytest.mark.parametrize("domain,dim,gravity", [("periodic", 3, None), ("reflect", 2, [0.0, -1.0]),
                                                ("reflect", 3, [0.0, 0.0, -2.0]), ("free", 3, None)])
def test_stages_replay_system_step(domain, dim, gravity):
    st, sy = make(domain, dim, gravity=gravity)
    n = 6
    want, wsy = jdem.System.step(st, sy, n=n)
    got, gsy = st, sy
    for _ in range(n):
        got, gsy = step_by_stages(got, gsy)
    for k in ("pos_c", "vel", "force"):
        assert np.array_equal(getattr(got, k), getattr(want, k)), k
    assert np.allclose(got.q.as_array(), want.q.as_array(), atol=2e-6)
    assert int(gsy.step_count) == int(wsy.step_count) == n
    if domain == "free":
        assert np.array_equal(gsy.domain.box_size, wsy.domain.box_size)
        assert np.array_equal(gsy.domain.anchor, wsy.domain.anchor)


def test_force_manager_stage_adds_external_forces_and_clears_them():
    st, sy = make("periodic", 3, N=256, gravity=[0.0, 0.0, -1.0])
    ext = np.random.default_rng(1).normal(size=st.force.shape).astype(F32)
    sy = jdem.ForceManager.add_force(st, sy, ext)
    sy = jdem.ForceManager.add_force(st, sy, 2 * ext, is_com=True)
    out, sy2 = sy.force_manager.apply(st, sy)
    g = np.array([0.0, 0.0, -1.0], F32)
    want = (st.force + ext) + (2 * ext + g * (st.mass / F32(1.0))[:, None])
    assert np.array_equal(out.force, want.astype(F32))
    assert not sy2.force_manager.external_force.any() and not sy2.force_manager.external_force_com.any()


def test_reflect_stage_bounces_a_sphere_off_the_wall():
    """One sphere moving into the x = 0 wall of a reflecting box comes back with the
    restitution's share of its speed (reflect.py:99-299, e = 1)."""
    st = jdem.State.create(pos=np.array([[0.49, 5.0, 5.0]], F32), vel=np.array([[-1.0, 0.0, 0.0]], F32),
                           rad=np.array([0.5], F32))
    sy = jdem.System.create(state=st, domain_type="reflect", dt=1e-3, domain_kw=dict(box_size=[10.0, 10.0, 10.0]))
    out, _ = sy.domain.apply(st, sy)
    assert out.vel[0, 0] > 0.0 and np.isclose(out.vel[0, 0], 1.0, rtol=1e-6)
    assert out.pos_c[0, 0] >= 0.49
