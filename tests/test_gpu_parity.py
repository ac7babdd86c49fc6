"""GPU parity: the sm_103a engine, through the C ABI, against the oracle.

Tolerances (from the benchmark specification):
  * contact pairs: bit-exact sorted (i < j) pairs;
  * forces: floored relative error <= 1e-5 in float32
    (err = max_i |dF_i| / max(|F_i|, 1e-3 rms|F|));
  * 100-step rollouts: <= 1e-4 position error (minimum image);
  * energy: the engine's total-energy trace equals the oracle's over 500 steps
    (test_gpu_dynamics.py); the Verlet energy-error slope > 1.8 is pinned on the
    float64 oracle (test_oracle_pins.py).
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
K = np.array([[1e3]], F32)


def small_periodic(N=2048, seed=7, phi=0.4, dim=3, radii=(0.5,)):
    rng = np.random.Generator(np.random.PCG64(seed))
    rad = rng.choice(np.asarray(radii), size=N)
    return W.periodic_system("t", rng, N, dim, rad, phi, 0.1, 1e-3, 100)


def reflect2d(N=2048, seed=8, phi=0.6):
    w = W.c3(N=N, seed=seed)
    return w


def free3d(N=1024, seed=9):
    w = small_periodic(N=N, seed=seed, phi=0.3)
    w.domain = "free"
    return w


def make_engine(w, skin=0.05, young=K, rotation="", **kw):
    d = w.desc()
    d["rotation"] = rotation
    d.update(kw)
    return Engine(w.dim, [d], young, skin=skin)


CASES = {
    "periodic3d": lambda: small_periodic(),
    "periodic2d": lambda: small_periodic(dim=2, phi=0.6),
    "bidisperse3d": lambda: small_periodic(radii=(0.5, 0.7), phi=0.55),
    "poly3_3d": lambda: small_periodic(radii=(0.2, 0.35, 0.6), phi=0.45),
    "tinybox3d": lambda: small_periodic(N=40, phi=0.4),
    "reflect2d": lambda: reflect2d(),
    "free3d": lambda: free3d(),
}


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


@pytest.mark.parametrize("case", list(CASES))
def test_compute_force_matches_oracle(case):
    w = CASES[case]()
    sy = osystem(w)
    st = ostate(w)
    ref64, _ = R.cell_list_force(st, sy, sum_dtype=np.float64)
    ref32, _ = R.cell_list_force(st, sy)
    eng = make_engine(w)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.compute_force()
        out = eng.download()
    finally:
        eng.close()
    e64 = force_err(out["force"], ref64)
    e32 = force_err(out["force"], ref32)
    g64 = global_force_err(out["force"], ref64)
    assert e64 <= 1e-5, f"{case}: err vs float64-accumulated oracle {e64}"
    assert e32 <= 1e-5, f"{case}: err vs float32 reference-order oracle {e32}"
    assert g64 <= 1e-5, f"{case}: ||dF|| / ||F|| vs float64-accumulated oracle {g64}"
    assert np.all(out["torque"] == 0)


@pytest.mark.parametrize("case", ["periodic3d", "periodic2d", "bidisperse3d", "reflect2d", "free3d", "tinybox3d"])
def test_contacts_bit_exact(case):
    w = CASES[case]()
    sy = osystem(w)
    st = ostate(w)
    ref = R.contact_pairs(st, sy)
    eng = make_engine(w)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        got = eng.contacts()
    finally:
        eng.close()
    assert got.shape == ref.shape, f"{case}: {got.shape} vs {ref.shape}"
    assert np.array_equal(got, ref)


def test_multi_material_force():
    w = small_periodic(N=2048, radii=(0.5, 0.6), phi=0.5)
    rng = np.random.default_rng(3)
    mat = rng.integers(0, 3, size=w.N).astype(np.int32)
    young = np.array([[1e3, 2e3, 5e2], [2e3, 4e3, 1e3], [5e2, 1e3, 2.5e2]], F32)
    sy = osystem(w, young=young)
    st = ostate(w, mat_id=mat)
    ref, _ = R.cell_list_force(st, sy, sum_dtype=np.float64)
    eng = make_engine(w, young=young)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel, mat_id=mat)
        eng.compute_force()
        out = eng.download()
    finally:
        eng.close()
    assert force_err(out["force"], ref) <= 1e-5


def test_excluded_pairs_bonds():
    """tests/test_excluded_pairs.py:11-61 on the device: bonds 0-1 and 1-2 are masked."""
    pos = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0]], F32)
    rad = np.full(3, 1.1, F32)
    bond = np.array([[1, -1], [0, 2], [1, -1]], np.int32)
    desc = dict(n=3, domain="free", linear="verlet", rotation="", dt=1e-3, box_size=[10, 10], anchor=[-5, -5],
                restitution=1.0, gravity=[0, 0], cell_size=2.2, search_range=1)
    eng = Engine(2, [desc], K, skin=0.0, bond_width=2)
    try:
        eng.upload(pos=pos, rad=rad, mass=np.ones(3, F32), bond_id=bond)
        eng.compute_force()
        f = eng.download()["force"]
    finally:
        eng.close()
    assert np.allclose(f[1], 0.0, atol=1e-5)
    assert abs(f[0, 0]) > 0.1 and abs(f[2, 0]) > 0.1
    assert np.allclose(f[0], -f[2], atol=1e-5)
    # k * (R - r) along the axis: 1e3 * (2.2 - 2.0) = 200
    assert np.isclose(abs(f[0, 0]), 200.0, rtol=1e-5)


@pytest.mark.parametrize("case,steps", [("periodic3d", 1), ("periodic3d", 100), ("periodic2d", 100),
                                        ("bidisperse3d", 100), ("reflect2d", 100), ("free3d", 100)])
def test_rollout_matches_oracle(case, steps):
    w = CASES[case]()
    if case == "reflect2d":
        w.vel = np.random.default_rng(1).normal(0, 0.5, size=w.vel.shape).astype(F32)
    pos, vel, frc = w.pos.copy(), w.vel.copy(), np.zeros_like(w.pos)
    box_o, anc_o = oracle.c_step(w.dim, pos, vel, frc, w.rad, w.mass, domain=w.domain, box=w.box_size,
                                 anchor=w.anchor, dt=w.dt, steps=steps, cell_size=2 * float(w.rad.max()),
                                 gravity=w.gravity, restitution=w.restitution, acc64=True)
    eng = make_engine(w)
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


def test_one_step_matches_numpy_reference_order():
    """One step from identical inputs against the float32 reference-order oracle."""
    w = small_periodic(N=1024)
    st = ostate(w)
    sy = osystem(w, rotation="verletspiral")
    st1, _ = R.step(st.copy(), sy, 1)
    eng = make_engine(w, rotation="verletspiral")
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.step(1)
        out = eng.download()
    finally:
        eng.close()
    assert force_err(out["force"], st1.force) <= 1e-5
    assert np.abs(out["pos_c"] - st1.pos_c).max() <= 1e-6
    assert np.array_equal(out["q"], st1.q)


def test_skin_does_not_change_forces():
    w = small_periodic(N=4096, radii=(0.5, 0.7), phi=0.55)
    outs = []
    for skin in (0.0, 0.05, 0.3):
        eng = make_engine(w, skin=skin)
        try:
            eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
            eng.step(30)
            outs.append(eng.download())
        finally:
            eng.close()
    for o in outs[1:]:
        assert min_image_diff(o["pos_c"], outs[0]["pos_c"], w.box_size) <= 1e-5
        assert force_err(o["force"], outs[0]["force"]) <= 1e-4


def test_energy_matches_oracle():
    w = small_periodic(N=2048, radii=(0.5, 0.7), phi=0.55)
    w2 = reflect2d(N=2048)
    for ww in (w, w2):
        st = ostate(ww)
        sy = osystem(ww)
        ref = R.compute_energy(st, sy)
        eng = make_engine(ww)
        try:
            eng.upload(pos=ww.pos, rad=ww.rad, mass=ww.mass, vel=ww.vel)
            e = eng.energy()
        finally:
            eng.close()
        assert np.allclose(e[:3], ref[:3], rtol=1e-5, atol=1e-6), (e, ref)


@pytest.mark.parametrize("dim,domain,radii", [(3, "periodic", (0.5,)), (2, "periodic", (0.5, 0.7)),
                                               (3, "reflect", (0.5,)), (3, "periodic", (0.1, 0.5))])
def test_neighbor_list_matches_reference_order(dim, domain, radii):
    w = small_periodic(N=512, dim=dim, radii=radii, phi=0.4)
    w.domain = domain
    sy = osystem(w)
    st = ostate(w)
    cutoff = 3.0 * float(w.rad.max())
    ref, ref_ovf = R.create_neighbor_list(st, sy, cutoff, 64)
    eng = make_engine(w, cell_size=float(sy.cell_size), search_range=max(int(np.max(sy.neighbor_mask)), 1))
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        nl, ovf = eng.neighbor_list(cutoff, 64)
    finally:
        eng.close()
    assert ovf == ref_ovf
    assert np.array_equal(nl, ref)


def test_batched_systems_match_alone():
    ws = [small_periodic(N=n, seed=s, phi=p, radii=(0.5, 0.7)) for n, s, p in ((300, 1, 0.35), (1500, 2, 0.5), (64, 3, 0.6))]
    eng = Engine(3, [w.desc() for w in ws], K, skin=0.05)
    try:
        eng.upload(pos=np.concatenate([w.pos for w in ws]), rad=np.concatenate([w.rad for w in ws]),
                   mass=np.concatenate([w.mass for w in ws]), vel=np.concatenate([w.vel for w in ws]))
        eng.step(100)
        batched = eng.download()
        e_b = eng.energy(per_system=True)
    finally:
        eng.close()
    off = 0
    for k, w in enumerate(ws):
        e1 = make_engine(w)
        try:
            e1.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
            e1.step(100)
            alone = e1.download()
            e_a = e1.energy()
        finally:
            e1.close()
        sl = slice(off, off + w.N)
        assert min_image_diff(batched["pos_c"][sl], alone["pos_c"], w.box_size) <= 1e-5
        assert force_err(batched["force"][sl], alone["force"]) <= 1e-4
        assert np.allclose(e_b[k], e_a, rtol=1e-4, atol=1e-6)
        off += w.N


def test_rotation_verlet_spiral_matches_oracle():
    w = small_periodic(N=512)
    rng = np.random.default_rng(5)
    ang = rng.normal(0, 2.0, size=(w.N, 3)).astype(F32)
    st = ostate(w, ang_vel=ang)
    sy = osystem(w, rotation="verletspiral")
    st1, _ = R.step(st.copy(), sy, 20)
    eng = make_engine(w, rotation="verletspiral")
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel, ang_vel=ang)
        eng.step(20)
        out = eng.download()
    finally:
        eng.close()
    assert np.allclose(out["q"], st1.q, atol=2e-6)
    assert np.allclose(out["ang_vel"], st1.ang_vel, rtol=1e-5, atol=1e-5)
    assert np.all(out["torque"] == 0)


@pytest.mark.parametrize("nl", [False, 4])
def test_verlet_list_paths_agree(nl):
    """Cell traversal every step (nl=False) and a list that overflows its initial
    capacity of 4 (cell traversal for those steps, then a larger list) match the
    default list path."""
    w = small_periodic(N=4096, radii=(0.5, 0.7), phi=0.55)
    outs = []
    for mode in (True, nl):
        eng = Engine(3, [w.desc()], K, skin=0.1, neighbor_list=mode)
        try:
            eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
            eng.step(60)
            outs.append(eng.download())
        finally:
            eng.close()
    assert min_image_diff(outs[1]["pos_c"], outs[0]["pos_c"], w.box_size) <= 1e-5
    assert force_err(outs[1]["force"], outs[0]["force"]) <= 1e-4


def test_unwrapped_periodic_positions_match_wrapped():
    """Periodic positions are never wrapped while stepping (domains/__init__.py:156-189):
    particles displaced by whole box lengths must see the same contacts and forces, and a
    rollout from such positions must follow the oracle run from the same positions."""
    w = small_periodic(N=4096, radii=(0.5, 0.7), phi=0.55, seed=31)
    rng = np.random.default_rng(4)
    shifted = (w.pos + rng.integers(-3, 4, size=w.pos.shape) * w.box_size).astype(F32)
    sy = osystem(w)
    st = ostate(w)
    st.pos_c = shifted
    ref, _ = R.cell_list_force(st, sy, sum_dtype=np.float64)
    st.pos_c = w.pos.copy()
    ref_wrapped, _ = R.cell_list_force(st, sy, sum_dtype=np.float64)
    eng = make_engine(w, skin=0.2)
    try:
        eng.upload(pos=shifted, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.compute_force()
        f0 = eng.download()["force"]
        eng.step(40)
        out = eng.download()
    finally:
        eng.close()
    assert force_err(f0, ref) <= 1e-5
    # against the wrapped configuration only to float32 cancellation in x_i - x_j at |x| ~ 4 boxes
    assert force_err(f0, ref_wrapped) <= 5e-3
    # the engine's first half-kick uses the force compute_force() stored; so does the oracle's
    pos, vel, frc = shifted.copy(), w.vel.copy(), np.asarray(ref, F32).copy()
    oracle.c_step(3, pos, vel, frc, w.rad, w.mass, domain="periodic", box=w.box_size, anchor=w.anchor,
                  dt=w.dt, steps=40, cell_size=2 * float(w.rad.max()), acc64=True)
    assert min_image_diff(out["pos_c"], pos, w.box_size) <= 1e-4


def _force_and_rollout(w, skin, steps=30):
    eng = Engine(w.dim, [w.desc()], K, skin=skin)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.compute_force()
        f0 = eng.download()["force"]
        eng.step(steps)
        out = eng.download()
        st = eng.stats()
    finally:
        eng.close()
    return f0, out, st


def _oracle_rollout(w, f0, steps=30):
    pos, vel, frc = w.pos.copy(), w.vel.copy(), np.asarray(f0, F32).copy()
    oracle.c_step(w.dim, pos, vel, frc, w.rad, w.mass, domain=w.domain, box=w.box_size, anchor=w.anchor,
                  dt=w.dt, steps=steps, cell_size=2 * float(w.rad.max()), acc64=True)
    return pos


def test_small_box_large_skin_keeps_minimum_image():
    """A skin so large against the box that a same-image pair could exceed half a box
    while the list lives: every list entry keeps the minimum image (grid of 3 cells)."""
    rng = np.random.Generator(np.random.PCG64(12))
    N = 165
    L = 6.0
    w = W.periodic_system("t", rng, N, 3, np.full(N, 0.5), 0.4, 0.5, 1e-3, 30)
    w.box_size = np.full(3, L, F32)
    w.pos = rng.uniform(0, L, (N, 3)).astype(F32)
    ref, _ = R.cell_list_force(ostate(w), osystem(w), sum_dtype=np.float64)
    f0, out, st = _force_and_rollout(w, skin=1.0)
    assert st["list_tiles"] > 0
    assert force_err(f0, ref) <= 1e-5
    assert min_image_diff(out["pos_c"], _oracle_rollout(w, ref), w.box_size) <= 1e-4


def test_clustered_particles_overflow_paths():
    """All particles in one corner of a large box: bricks whose stencil region exceeds
    the shared-memory staging build from global memory, and rows longer than the initial
    capacity fall back to the cell traversal until the capacity grows."""
    rng = np.random.Generator(np.random.PCG64(13))
    N = 3000
    w = W.periodic_system("t", rng, N, 3, rng.choice([0.5, 0.7], N), 0.05, 0.1, 5e-4, 30)
    w.pos = rng.uniform(0, 0.2 * float(w.box_size[0]), (N, 3)).astype(F32)
    ref, _ = R.cell_list_force(ostate(w), osystem(w), sum_dtype=np.float64)
    f0, out, st = _force_and_rollout(w, skin=0.3)
    assert st["list_tiles"] > 0
    assert force_err(f0, ref) <= 1e-5
    assert min_image_diff(out["pos_c"], _oracle_rollout(w, ref), w.box_size) <= 1e-4


def test_upload_rejects_bad_input_and_recovers():
    """Non-finite positions, negative radii and material ids outside the table are
    rejected at upload (checked on the device); the handle then holds no state until
    an upload succeeds."""
    from jaxdem_gb300._lib import JdemError

    w = small_periodic(N=1024)
    eng = make_engine(w)
    try:
        bad = w.pos.copy()
        bad[17, 1] = np.nan
        with pytest.raises(JdemError) as e:
            eng.upload(pos=bad, rad=w.rad, mass=w.mass, vel=w.vel)
        assert "non-finite" in str(e.value)
        with pytest.raises(JdemError):
            eng.step(1)
        rad = w.rad.copy()
        rad[3] = -0.5
        with pytest.raises(JdemError):
            eng.upload(pos=w.pos, rad=rad, mass=w.mass, vel=w.vel)
        mat = np.zeros(w.N, np.int32)
        mat[5] = 7
        with pytest.raises(JdemError):
            eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel, mat_id=mat)
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.step(10)
        out = eng.download()
    finally:
        eng.close()
    ref = make_engine(w)
    try:
        ref.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        ref.step(10)
        want = ref.download()
    finally:
        ref.close()
    assert np.array_equal(out["pos_c"], want["pos_c"])
