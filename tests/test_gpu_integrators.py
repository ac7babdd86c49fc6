"""Integrator stages through the split factory types (``jdem_integrate``).

``LinearIntegrator.create(key).step_before_force / step_after_force`` and the
rotation integrators' stages run on the GPU and are held against the oracle's
restatement of each stage (velocity_verlet.py:29-95, direct_euler.py:30-66,
velocity_verlet_spiral.py:36-180, spiral.py:56-144) on random states with
fixed particles and torques: positions and velocities bit for bit, q and
angular velocity to 2e-6.
"""

from __future__ import annotations

import numpy as np
import pytest

from jaxdem_gb300 import State
from jaxdem_gb300.integrators import LinearIntegrator, RotationIntegrator
from oracle import dem_ref as R

pytestmark = pytest.mark.gpu

F32 = np.float32


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


class _Sys:
    def __init__(self, dt):
        self.dt = F32(dt)


def _random(dim, n=5000, seed=0):
    rng = np.random.default_rng(seed)
    ad = 3 if dim == 3 else 1
    q = rng.normal(size=(n, 4)).astype(F32)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    arrays = dict(pos=rng.uniform(-5, 5, (n, dim)).astype(F32), vel=rng.normal(0, 1, (n, dim)).astype(F32),
                  force=rng.normal(0, 30, (n, dim)).astype(F32), mass=rng.uniform(0.2, 2.0, n).astype(F32),
                  fixed=rng.random(n) < 0.1, ang_vel=rng.normal(0, 2, (n, ad)).astype(F32),
                  torque=rng.normal(0, 5, (n, ad)).astype(F32), inertia=rng.uniform(0.05, 1.0, (n, ad)).astype(F32),
                  q=q)
    st = State.create(pos=arrays["pos"], vel=arrays["vel"], force=arrays["force"], mass=arrays["mass"],
                      fixed=arrays["fixed"], ang_vel=arrays["ang_vel"], torque=arrays["torque"],
                      inertia=arrays["inertia"], q=q)
    ost = R.make_state(arrays["pos"], vel=arrays["vel"], mass=arrays["mass"], fixed=arrays["fixed"],
                       ang_vel=arrays["ang_vel"], torque=arrays["torque"], q=q, force=arrays["force"],
                       inertia=arrays["inertia"])
    return st, ost


LINEAR_CASES = [("verlet", 0, R.vv_before), ("verlet", 1, R.vv_after), ("euler", 1, R.euler_after),
                ("euler", 0, None)]
ROTATION_CASES = [("verletspiral", 0, R.vvspiral_before), ("verletspiral", 1, R.vvspiral_after),
                  ("spiral", 1, R.spiral_after), ("spiral", 0, None)]


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("key,stage,ref", LINEAR_CASES)
def test_linear_stage_matches_the_oracle(dim, key, stage, ref):
    st, ost = _random(dim, seed=dim * 10 + stage)
    integ = LinearIntegrator.create(key)
    fn = integ.step_before_force if stage == 0 else integ.step_after_force
    out, _ = fn(st, _Sys(1e-3))
    want = ost if ref is None else ref(ost, _Sys(1e-3))
    assert np.array_equal(out.pos_c, want.pos_c)
    assert np.array_equal(out.vel, want.vel)
    assert np.array_equal(out.q.as_array(), st.q.as_array())  # linear stages leave rotation alone
    if ref is not None:
        assert not np.array_equal(out.vel, st.vel)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("key,stage,ref", ROTATION_CASES)
def test_rotation_stage_matches_the_oracle(dim, key, stage, ref):
    st, ost = _random(dim, seed=100 + dim * 10 + stage)
    integ = RotationIntegrator.create(key)
    fn = integ.step_before_force if stage == 0 else integ.step_after_force
    out, _ = fn(st, _Sys(2e-3))
    want = ost if ref is None else ref(ost, _Sys(2e-3))
    assert np.allclose(out.q.as_array(), want.q, rtol=0, atol=2e-6)
    assert np.allclose(out.ang_vel, want.ang_vel, rtol=2e-6, atol=2e-6)
    assert np.array_equal(out.pos_c, st.pos_c) and np.array_equal(out.vel, st.vel)


def test_batched_state_uses_each_systems_dt():
    st, _ = _random(3, n=1000, seed=7)
    bst = State.stack([st, st])
    sysb = _Sys(0.0)
    sysb.dt = np.array([1e-3, 2e-3], F32)
    out, _ = LinearIntegrator.create("verlet").step_before_force(bst, sysb)
    for b, dt in enumerate((1e-3, 2e-3)):
        one, _ = LinearIntegrator.create("verlet").step_before_force(st, _Sys(dt))
        assert np.array_equal(out.pos_c[b], one.pos_c)
