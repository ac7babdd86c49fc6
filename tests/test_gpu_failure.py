"""Failure paths of the engine, made on the host with valid inputs (no GPU fault).

* A state that blows up during the steps (host-chosen masses so small that the first
  contact forces throw the spheres past the float32 range) is reported by jdem_step as
  JDEM_ERR_NONFINITE, on the many-step path of small systems and on direct launches;
  the handle then takes a fresh upload and steps exactly like a new handle.
* The many-step kernel's grid barrier is bounded: with extra arrivals that never come
  (jdem_set_barrier_limit) every block gives up after its poll limit, the kernel
  returns, jdem_step reports JDEM_ERR_TIMEOUT, and the handle continues on per-step
  launches whose results equal a direct-launch handle's bit for bit.
"""

from __future__ import annotations

import numpy as np
import pytest

from jaxdem_gb300 import workloads as W
from jaxdem_gb300._lib import Engine, JdemError

pytestmark = pytest.mark.gpu

K = np.array([[W.K_SPRING]], np.float32)
ERR_NONFINITE = 4
ERR_TIMEOUT = 6


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def _steps(w, n, **kw):
    eng = Engine(w.dim, [w.desc()], K, skin=0.3, **kw)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.step(n)
        return eng.download()
    finally:
        eng.close()


@pytest.mark.parametrize("graph_mode", [0, 2])
def test_blow_up_mid_run_reports_nonfinite_and_recovers(graph_mode):
    w = W.c1(N=2048, seed=41)
    tiny = np.full(w.N, 1e-30, np.float32)
    eng = Engine(3, [w.desc()], K, skin=0.3, graph_mode=graph_mode)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=tiny, vel=w.vel)  # finite inputs: accepted
        with pytest.raises(JdemError) as e:
            eng.step(6)
        assert e.value.code == ERR_NONFINITE
        assert "non-finite" in str(e.value)
        # a fresh upload clears the state; the handle steps like a new one
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.step(25)
        out = eng.download()
        assert eng.stats()["device_status"] == 0
    finally:
        eng.close()
    want = _steps(w, 25, graph_mode=graph_mode)
    assert np.array_equal(out["pos_c"], want["pos_c"])
    assert np.array_equal(out["vel"], want["vel"])


def test_barrier_timeout_reports_timeout_then_runs_per_step():
    w = W.c1(N=2048, seed=42)
    eng = Engine(3, [w.desc()], K, skin=0.3)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.step(20)
        assert eng.stats()["many_step"] == 1, "this small system should take the many-step path"
        eng.set_barrier_limit(2000, 1)  # one arrival that never comes: every barrier gives up
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        with pytest.raises(JdemError) as e:
            eng.step(20)
        assert e.value.code == ERR_TIMEOUT
        assert "barrier" in str(e.value)
        st = eng.stats()
        assert st["many_step"] == 0 and st["device_status"] == 0
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.step(30)
        out = eng.download()
        assert eng.stats()["many_step"] == 0
    finally:
        eng.close()
    want = _steps(w, 30, graph_mode=2)
    assert np.array_equal(out["pos_c"], want["pos_c"])
    assert np.array_equal(out["vel"], want["vel"])
