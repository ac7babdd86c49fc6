"""GPU parity at the benchmark configurations' full sizes, through the C ABI, against
the C/OpenMP oracle (float64 force accumulation).

  * 1,048,576 bidisperse spheres, periodic, packing fraction 0.55 (the bench workload):
    step-0 forces (floored relative error and ||dF|| / ||F|| <= 1e-5), contact pairs
    bit-exact, one step, and a 20-step rollout <= 1e-4 in position;
  * 4,194,304 polydisperse disks in a reflecting box with gravity: the same checks over
    10 steps;
  * 4096 monodisperse spheres for the configured 1000 steps: positions <= 1e-4 and the
    total-energy trace (every 100 steps) against the oracle's;
  * 96 systems of the batched configuration's size and density distribution in one
    handle, each held against the oracle run on it alone.

These runs take the code paths only large grids take (thousands of list-build bricks,
87^3 and 1820^2 binning grids, list-capacity planning at full density), which the
small-case parity tests never reach.  Size-independent checks ride along: with no
gravity the contact forces of a periodic system sum to zero (Newton's third law of the
spring, forces/spring.py:97-108), so total momentum stays constant.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from jaxdem_gb300 import workloads as W
from jaxdem_gb300._lib import Engine
from oracle import dem_ref as R
from tests.helpers import force_err, global_force_err, min_image_diff, osystem, ostate

pytestmark = pytest.mark.gpu

F32 = np.float32
K = np.array([[W.K_SPRING]], F32)
SKIN_OVER_RMAX = 0.65  # the engine's default skin for these workloads


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def _okw(w):
    return dict(domain=w.domain, box=w.box_size, anchor=w.anchor, cell_size=2 * float(w.rad.max()))


def _engine(w, **kw):
    return Engine(w.dim, [w.desc()], K, skin=SKIN_OVER_RMAX * float(w.rad.max()), **kw)


def _check_force_contacts_rollout(w, steps):
    ref_f = oracle.c_force(w.dim, w.pos, w.rad, acc64=True, **_okw(w))
    ref_pairs = oracle.c_contacts(w.dim, w.pos, w.rad, **_okw(w))
    pos1, vel1, frc1 = w.pos.copy(), w.vel.copy(), np.zeros_like(w.pos)
    oracle.c_step(w.dim, pos1, vel1, frc1, w.rad, w.mass, dt=w.dt, steps=1, gravity=w.gravity,
                  restitution=w.restitution, acc64=True, **_okw(w))
    pos, vel, frc = pos1.copy(), vel1.copy(), frc1.copy()
    box_o, anc_o = oracle.c_step(w.dim, pos, vel, frc, w.rad, w.mass, dt=w.dt, steps=steps - 1,
                                 gravity=w.gravity, restitution=w.restitution, acc64=True, **_okw(w))
    eng = _engine(w)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.compute_force()
        f0 = eng.download()["force"]
        pairs = eng.contacts()
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.step(1)
        one = eng.download()
        eng.step(steps - 1)
        out = eng.download()
        st = eng.stats()
    finally:
        eng.close()
    per_box = w.box_size if w.domain == "periodic" else None
    e_f, g_f = force_err(f0, ref_f), global_force_err(f0, ref_f)
    assert e_f <= 1e-5, f"step-0 force: floored relative error {e_f}"
    assert g_f <= 1e-5, f"step-0 force: ||dF|| / ||F|| = {g_f}"
    assert pairs.shape == ref_pairs.shape, f"contact count {len(pairs)} vs oracle {len(ref_pairs)}"
    assert np.array_equal(pairs, ref_pairs), "contact pairs differ from the oracle's"
    assert min_image_diff(one["pos_c"], pos1, per_box) <= 1e-5
    assert force_err(one["force"], frc1) <= 1e-5
    d = min_image_diff(out["pos_c"], pos, per_box)
    assert d <= 1e-4, f"{steps}-step rollout: position error {d}"
    assert force_err(out["force"], frc) <= 1e-3
    assert st["list_tiles"] > 1000, "the full-size grid should plan thousands of list-build bricks"
    return f0, out, st


def test_c2_full_size_force_contacts_rollout():
    """1,048,576 spheres (the bench workload), 20 steps."""
    w = W.c2()
    f0, out, st = _check_force_contacts_rollout(w, steps=20)
    # Newton's third law: the contact forces of a periodic system without gravity cancel
    f64 = f0.astype(np.float64)
    assert np.abs(f64.sum(0)).max() <= 1e-6 * np.abs(f64).sum(0).max()
    p0 = (w.mass[:, None].astype(np.float64) * w.vel).sum(0)
    p1 = (w.mass[:, None].astype(np.float64) * out["vel"]).sum(0)
    scale = (w.mass[:, None].astype(np.float64) * np.abs(out["vel"])).sum(0).max()
    assert np.abs(p1 - p0).max() <= 1e-5 * scale


def test_c3_full_size_force_contacts_rollout():
    """4,194,304 disks, reflecting walls and gravity, 10 steps."""
    w = W.c3()
    _check_force_contacts_rollout(w, steps=10)


def test_c1_as_configured_1000_steps():
    """4096 spheres for the configured 1000 steps: positions against the oracle and the
    total-energy trace (collider PE + KE; spring law, periodic, no gravity) every 100 steps."""
    w = W.c1()
    assert w.steps == 1000
    stride, n_frames = 100, w.steps // 100
    pos, vel, frc = w.pos.copy(), w.vel.copy(), np.zeros_like(w.pos)
    sy = osystem(w)
    ref_e, ref_pos = [], []
    for _ in range(n_frames):
        oracle.c_step(3, pos, vel, frc, w.rad, w.mass, dt=w.dt, steps=stride, acc64=True, **_okw(w))
        st = ostate(w)
        st.pos_c, st.vel = pos.copy(), vel.copy()
        ref_e.append(R.compute_energy(st, sy)[:3])
        ref_pos.append(pos.copy())
    eng = _engine(w)
    gpu_e = []
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        for t in range(n_frames):
            eng.step(stride)
            gpu_e.append(eng.energy()[:3])
            out = eng.download()
            d = min_image_diff(out["pos_c"], ref_pos[t], w.box_size)
            assert d <= 1e-4, f"after {(t + 1) * stride} steps: position error {d}"
    finally:
        eng.close()
    gpu_e, ref_e = np.asarray(gpu_e), np.asarray(ref_e)
    tot_g, tot_r = gpu_e.sum(1), ref_e.sum(1)
    assert np.allclose(tot_g, tot_r, rtol=1e-5, atol=1e-6), (tot_g, tot_r)
    assert np.allclose(gpu_e, ref_e, rtol=1e-4, atol=1e-5)


def test_c4_style_uneven_batch_against_the_oracle(steps=100):
    """Systems of the batched configuration's distribution (log-uniform sizes, packing
    fractions 0.30-0.60, bidisperse radii, periodic boxes), stepped together in one handle
    (per-system parameters and cell segments) and each held directly against the C oracle
    run on that system alone: positions <= 1e-4 after 100 steps, forces <= 1e-3, and the
    per-system energies of the final state to 1e-5 of the oracle's energies of that state."""
    ws = W.c4(n_systems=96, seed=44, n_min=64, n_max=8192)
    eng = Engine(3, [w.desc() for w in ws], K, skin=SKIN_OVER_RMAX * 0.7)
    try:
        eng.upload(pos=np.concatenate([w.pos for w in ws]), rad=np.concatenate([w.rad for w in ws]),
                   mass=np.concatenate([w.mass for w in ws]), vel=np.concatenate([w.vel for w in ws]))
        eng.step(steps)
        out = eng.download()
        e = eng.energy(per_system=True)
    finally:
        eng.close()
    off = 0
    worst = 0.0
    for k, w in enumerate(ws):
        pos, vel, frc = w.pos.copy(), w.vel.copy(), np.zeros_like(w.pos)
        oracle.c_step(3, pos, vel, frc, w.rad, w.mass, dt=w.dt, steps=steps, acc64=True, **_okw(w))
        sl = slice(off, off + w.N)
        d = min_image_diff(out["pos_c"][sl], pos, w.box_size)
        worst = max(worst, d)
        assert d <= 1e-4, f"system {k} (N={w.N}): position error {d}"
        assert force_err(out["force"][sl], frc) <= 1e-3, f"system {k}: force"
        st = R.make_state(out["pos_c"][sl], vel=out["vel"][sl], rad=w.rad, mass=w.mass)
        ref = R.compute_energy(st, osystem(w))
        assert np.allclose(e[k][0], ref[0], rtol=1e-5, atol=1e-7), f"system {k}: contact energy"
        assert np.allclose(e[k][2], ref[2], rtol=1e-5, atol=1e-7), f"system {k}: kinetic energy"
        off += w.N
    print(f"C4-style batch of {len(ws)} systems ({off} spheres): worst position error {worst:.2e}")
