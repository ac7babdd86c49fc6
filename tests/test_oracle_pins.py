"""Pin the oracle (CPU restatement) against the reference's own known answers.

JaxDEM cannot run here (no JAX), and it ships no golden arrays; these tests
restate the reference tests that pin the hot path, plus hand-derived
analytic cases, on the numpy and C restatements:

* ``tests/test_excluded_pairs.py:11-61``: bonded pairs are masked, F1 = 0, F0 = -F2;
* ``tests/test_colliders_invariance.py:365-402``: the cell list equals the all-pairs sum;
* ``tests/test_energy_conservation.py:34-107``: Verlet energy-error slope > 1.8,
  Euler > 0.7, spheres in periodic / reflect / free domains, 2D and 3D;
* ``tests/test_rotation_integrators.py:24-97``: torque-driven asymmetric body
  against the closed form, relative error < 1e-4;
* two overlapping spheres (|F| = k delta), a periodic image pair, a wall bounce;
* the Hertz law (no reference test covers it): two spheres against the closed
  form, F = -dE/dd, and the C restatement against numpy;
* the Cundall-Strack law (no reference test covers it either): damping, sliding
  friction below and at the Coulomb cap, torques, rolling friction, 2D and 3D.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from jaxdem_gb300 import workloads as W
from oracle import dem_ref as R

F32 = np.float32


def _sys(dim, domain="periodic", box=None, anchor=None, rad=None, young=1e3, dt=1e-3, gravity=None,
         linear="verlet", rotation="", dtype=F32):
    cell, mask = R.cell_list_create(rad, dim, dtype=dtype)
    box = np.full(dim, 10.0, dtype) if box is None else np.asarray(box, dtype)
    anchor = np.zeros(dim, dtype) if anchor is None else np.asarray(anchor, dtype)
    return R.OSystem(dim=dim, domain=domain, box_size=box, anchor=anchor,
                     young_eff=np.array([[young]], dtype), dt=dtype(dt), cell_size=cell, neighbor_mask=mask,
                     gravity=np.zeros(dim, dtype) if gravity is None else np.asarray(gravity, dtype),
                     linear=linear, rotation=rotation)


def test_excluded_pairs():
    """tests/test_excluded_pairs.py:11-61 on the restatement (cell list and all pairs)."""
    pos = np.array([[0.0, 0.0], [1.0, 0.0], [2.0, 0.0]], F32)
    rad = np.full(3, 1.1, F32)
    bond = np.array([[1, -1], [0, 2], [1, -1]])
    st = R.make_state(pos, rad=rad, bond_id=bond)
    # linear matcher of one material: young_eff = young = 1000
    sy = _sys(2, domain="free", box=[1, 1], rad=rad)
    for f in (R.cell_list_force(st, sy)[0], R.naive_force(st, sy)):
        assert np.allclose(f[1], 0.0, atol=1e-5)
        assert abs(f[0, 0]) > 0.1 and abs(f[2, 0]) > 0.1
        assert np.allclose(f[0], -f[2], atol=1e-5)


def test_two_sphere_spring_analytic():
    """F = k delta r_hat (spring.py:97-108), E = k delta^2 / 2 per pair."""
    k, r0, r1, d = 1e3, 0.5, 0.7, 1.0
    pos = np.array([[1.0, 2.0, 3.0], [1.0 + d, 2.0, 3.0]], F32)
    rad = np.array([r0, r1], F32)
    st = R.make_state(pos, rad=rad)
    sy = _sys(3, domain="free", rad=rad, young=k)
    f, _ = R.cell_list_force(st, sy, sum_dtype=np.float64)
    delta = r0 + r1 - d
    assert np.allclose(f[0], [-k * delta, 0, 0], rtol=1e-6)
    assert np.allclose(f[1], [k * delta, 0, 0], rtol=1e-6)
    assert np.isclose(R.cell_list_energy(st, sy), 0.5 * k * delta ** 2, rtol=1e-6)


def test_two_sphere_hertz_analytic():
    """Hertz law (forces/hertz.py:22-170), hand-derived: 1/E* = 2 (1 - nu^2) / E for two
    spheres of one material, R* = r0 r1 / (r0 + r1), k = (4/3) E* sqrt(R*),
    |F| = k delta^(3/2) along r_hat, E = (2/5) k delta^(5/2); and F = -dE/dd by a
    central difference of the float64 oracle."""
    E, nu, r0, r1 = 1e3, 0.3, 0.5, 0.7
    k43 = R.hertz_constant([E], [nu])
    assert np.isclose(k43[0, 0], 4.0 / 3.0 * E / (2 * (1 - nu * nu)), rtol=1e-6)
    k = 4.0 / 3.0 * E / (2 * (1 - nu * nu)) * np.sqrt(r0 * r1 / (r0 + r1))
    rad = np.array([r0, r1], F32)

    def hertz_sys(dtype):
        s = _sys(3, domain="free", rad=rad, dtype=dtype)
        s.young_eff = k43.astype(dtype)
        s.force_law = "hertz"
        return s

    for d in (1.0, 1.1, 1.19):
        pos = np.array([[1.0, 2.0, 3.0], [1.0 + d, 2.0, 3.0]], F32)
        st = R.make_state(pos, rad=rad)
        f, _ = R.cell_list_force(st, hertz_sys(F32), sum_dtype=np.float64)
        # the overlap of the stored float32 radii and coordinates; float32 R - r loses
        # about one ulp of r (1.2e-7 r) to cancellation, amplified 3/2 by delta^(3/2)
        delta = float(rad[0]) + float(rad[1]) - (float(pos[1, 0]) - float(pos[0, 0]))
        tol = 2e-6 + 3.0 * 1.2e-7 * d / delta
        assert np.allclose(f[0], [-k * delta ** 1.5, 0, 0], rtol=tol)
        assert np.allclose(f[1], [k * delta ** 1.5, 0, 0], rtol=tol)
        assert np.isclose(R.cell_list_energy(st, hertz_sys(F32)), 0.4 * k * delta ** 2.5, rtol=2 * tol)
        assert np.allclose(R.naive_force(st, hertz_sys(F32)), f, rtol=1e-6)
    # the force is minus the energy gradient (float64 oracle)
    sy64 = hertz_sys(np.float64)
    d, h = 1.05, 1e-6

    def energy(dd):
        p = np.array([[1.0, 2.0, 3.0], [1.0 + dd, 2.0, 3.0]])
        return R.cell_list_energy(R.make_state(p, rad=rad, dtype=np.float64), sy64)

    p = np.array([[1.0, 2.0, 3.0], [1.0 + d, 2.0, 3.0]])
    f64, _ = R.cell_list_force(R.make_state(p, rad=rad, dtype=np.float64), sy64)
    assert np.isclose(f64[1, 0], -(energy(d + h) - energy(d - h)) / (2 * h), rtol=1e-6)
    # apart: no force
    st = R.make_state(np.array([[0.0, 0, 0], [1.3, 0, 0]], F32), rad=rad)
    assert not np.any(R.cell_list_force(st, hertz_sys(F32))[0])


def test_hertz_c_restatement_matches_numpy():
    """The C/OpenMP Hertz law against the numpy oracle on a polydisperse, two-material
    periodic packing: agreement to the last bits of pow (different libm routines)."""
    rng = np.random.Generator(np.random.PCG64(31))
    N, L = 2000, 13.0
    pos = rng.uniform(0, L, (N, 3)).astype(F32)
    rad = rng.choice([0.5, 0.6, 0.7], N).astype(F32)
    mat = rng.integers(0, 2, N).astype(np.int32)
    k43 = R.hertz_constant([1e3, 4e3], [0.3, 0.2])
    st = R.make_state(pos, rad=rad, mat_id=mat)
    sy = _sys(3, domain="periodic", box=[L] * 3, rad=rad)
    sy.young_eff, sy.force_law = k43, "hertz"
    f, _ = R.cell_list_force(st, sy, sum_dtype=np.float64)
    fc = oracle.c_force(3, pos, rad, domain="periodic", box=sy.box_size, anchor=sy.anchor,
                        cell_size=float(sy.cell_size), young=k43, mat_id=mat, acc64=True, law="hertz")
    scale = np.abs(f).max()
    assert scale > 0 and np.abs(f - fc).max() <= 1e-6 * scale


def _cs_sys(st, e=0.5, mu=0.4, mu_r=0.0, young=1e3, poisson=0.25, dtype=np.float64):
    sy = _sys(3, domain="free", rad=st.rad, dtype=dtype)
    beta, props = R.cs_tables([young], [poisson], [e], [mu], [mu_r])
    sy.young_eff, sy.mat_props, sy.force_law = beta.astype(dtype), props.astype(dtype), "cundallstrack"
    return sy


def test_cundall_strack_closed_forms():
    """Cundall-Strack (forces/cundall_strack.py:22-242), hand-derived on two equal spheres
    (radius R, mass m, one material; no reference test covers the law):
    kn = E R, m_eff = m / 2, beta = -ln e / sqrt(pi^2 + ln^2 e), gamma = 2 beta sqrt(k m_eff);
    head-on approach: F = (kn delta - gamma_n vn) n; sliding: a tangential force of
    min(gamma_t |v_t|, mu Fn) against the slip and a torque R Ft about n x t; e = 1: no
    damping; rolling friction: a torque mu_r R_eff Fn against the relative spin."""
    E, nu, Rr, m, e, mu = 1e3, 0.25, 0.5, 2.0, 0.5, 0.4
    G = E / (2 * (1 + nu))
    beta = -np.log(e) / np.sqrt(np.pi ** 2 + np.log(e) ** 2)
    # the material tables are float32 (as in the reference): compare to 1e-6
    kn, kt, m_eff = E * Rr, G * Rr, m / 2
    gn, gt = 2 * beta * np.sqrt(kn * m_eff), 2 * beta * np.sqrt(kt * m_eff)
    d, delta = 0.9, 0.1

    def state(vel, w=None):
        st = R.make_state(np.array([[0.0, 0, 0], [-d, 0, 0]]), rad=[Rr, Rr], mass=[m, m],
                          vel=np.asarray(vel, float), dtype=np.float64)
        if w is not None:
            st.ang_vel = np.asarray(w, np.float64)
        return st

    # head-on: i moves towards j at 0.3 (n = +x points from j to i, vn = -0.3)
    st = state([[-0.3, 0, 0], [0, 0, 0]])
    f, t = R.cell_list_force(st, _cs_sys(st))
    assert np.allclose(f[0], [kn * delta + gn * 0.3, 0, 0], rtol=1e-6)
    assert np.allclose(f[1], -f[0], rtol=1e-6) and not np.any(t)
    # sliding along y at 0.2: dashpot below the Coulomb cap, torque about z
    st = state([[0, 0.2, 0], [0, 0, 0]])
    f, t = R.cell_list_force(st, _cs_sys(st, mu=10.0))
    ft = gt * 0.2
    assert np.allclose(f[0], [kn * delta, -ft, 0], rtol=1e-6)
    # r_ci = -R n = (-R, 0, 0); torque = r_ci x F = (0, 0, R ft)
    assert np.allclose(t[0], [0, 0, Rr * ft], rtol=1e-6)
    # a fast slide saturates at mu Fn
    st = state([[0, 50.0, 0], [0, 0, 0]])
    f, _ = R.cell_list_force(st, _cs_sys(st))
    assert np.isclose(-f[0, 1], mu * kn * delta, rtol=1e-6)
    # e = 1: no damping at all, the spring of stiffness kn remains
    st = state([[-0.3, 0.2, 0], [0, 0, 0]])
    f, _ = R.cell_list_force(st, _cs_sys(st, e=1.0))
    assert np.allclose(f[0], [kn * delta, 0, 0], atol=1e-9)
    # rolling friction opposes the relative spin about n (which adds no contact-point slip)
    st = state([[0, 0, 0], [0, 0, 0]], w=[[3.0, 0, 0], [0, 0, 0]])
    _, t = R.cell_list_force(st, _cs_sys(st, mu_r=0.2))
    assert np.allclose(t[0], [-0.2 * (Rr / 2) * kn * delta, 0, 0], rtol=1e-6)
    # energy 0.5 kn delta^2 per pair
    assert np.isclose(R.cell_list_energy(st, _cs_sys(st)), 0.5 * kn * delta ** 2, rtol=1e-6)


def test_cundall_strack_spin_slip_and_2d():
    """A spinning sphere on a resting one: the contact point of i moves at w x r_ci, so a
    spin about z of i slides the contact along -y (3D); in 2D the same contact gives the
    scalar torque, and the float32 oracle follows the float64 one."""
    E, Rr, m = 1e3, 0.5, 2.0
    for dim in (3, 2):
        pos = np.array([[0.0] * dim, [-0.9] + [0.0] * (dim - 1)])
        w = np.zeros((2, 3 if dim == 3 else 1))
        w[0, -1] = 2.0
        out = {}
        for dtype in (np.float64, F32):
            st = R.make_state(pos, rad=[Rr, Rr], mass=[m, m], dtype=dtype)
            st.ang_vel = w.astype(dtype)
            sy = _sys(dim, domain="free", rad=st.rad, dtype=dtype)
            beta, props = R.cs_tables([E], [0.25], [0.5], [10.0], [0.0])
            sy.young_eff, sy.mat_props, sy.force_law = beta.astype(dtype), props.astype(dtype), "cundallstrack"
            out[dtype] = R.cell_list_force(st, sy)
        f, t = out[np.float64]
        # w x r_ci with r_ci = (-R, 0) and w = 2 e_z: (0, -2R); friction acts along +y
        assert f[0, 1] > 0 and np.isclose(f[0, 1], -f[1, 1])
        # torque on i: r_ci x F = -R * F_y about z, opposing the spin
        assert np.isclose(t[0, -1], -Rr * f[0, 1], rtol=1e-9) and t[0, -1] < 0
        f32, t32 = out[F32]
        assert np.allclose(f32, f, rtol=1e-5, atol=1e-6) and np.allclose(t32, t, rtol=1e-5, atol=1e-6)


def test_rigid_clump_closed_forms():
    """Rigid clumps (State.add_clump, state.py:1230-1420; ForceManager.apply,
    force_manager.py:338-425): overlapping members of one clump exert nothing on each
    other (colliders/__init__.py:225-243); contact forces between two clumps balance; a
    contact at a member's offset r gives the clump the torque r x F about its centre;
    gravity gives every member M g after the clump sum and no torque."""
    f64 = np.float64
    # two dumbbells along x: members at the centre +- (0.4, 0, 0), radius 0.5 (the members
    # of one clump overlap by 0.2); clump B's left sphere overlaps clump A's right one
    pc = np.array([[0.0, 0, 0], [0.0, 0, 0], [1.7, 0.3, 0], [1.7, 0.3, 0]])
    pp = np.array([[-0.4, 0, 0], [0.4, 0, 0], [-0.4, 0, 0], [0.4, 0, 0]])
    M, I = 2.0, [1.0, 1.0, 1.0]
    st = R.make_state(pc, rad=[0.5] * 4, mass=[M] * 4, inertia=[I] * 4, pos_p=pp, clump_id=[0, 0, 1, 1],
                      dtype=f64)
    sy = _sys(3, domain="free", rad=st.rad, young=1e3, dtype=f64, gravity=[0, -9.8, 0])
    f, t = R.cell_list_force(st, sy)
    # only the A1-B0 pair touches across clumps: d = (1.7 - 0.4) - 0.4 = 0.9 along x, 0.3 along y
    d = np.array([0.9, 0.3, 0.0])
    r = np.linalg.norm(d)
    fab = 1e3 * (1.0 - r) * d / r  # force on B0 from A1
    assert np.allclose(f[0], 0) and np.allclose(f[3], 0)
    assert np.allclose(f[2], fab, rtol=1e-12) and np.allclose(f[1], -fab, rtol=1e-12)
    # torques about each clump centre: r x F with r = +-0.4 x
    assert np.allclose(t[1], np.cross([0.4, 0, 0], -fab), rtol=1e-12)
    assert np.allclose(t[2], np.cross([-0.4, 0, 0], fab), rtol=1e-12)
    st.force, st.torque = f, t
    st = R.force_manager_apply(st, sy)
    g = np.array([0.0, -9.8, 0.0])
    assert np.allclose(st.force[:2], -fab + M * g, rtol=1e-12) and np.allclose(st.force[2:], fab + M * g, rtol=1e-12)
    assert np.allclose(st.torque[:2], np.cross([0.4, 0, 0], -fab)) and np.allclose(st.torque[2:], np.cross([-0.4, 0, 0], fab))
    # the momentum exchanged balances
    assert np.allclose(st.force[0] + st.force[2], 2 * M * g)
    # contact set: the overlapping members of one clump are not contacts
    assert R.contact_pairs(st, sy).tolist() == [[1, 2]]


def test_rigid_clump_free_box_and_step():
    """FreeDomain.apply with clumps (free.py:59-63) bounds pos_c -+ (|pos_p| + rad); a lone
    spinning clump keeps its shape and centre velocity through the integrators."""
    f64 = np.float64
    pc = np.array([[1.0, 2.0, 3.0]] * 3)
    pp = np.array([[0.3, 0, 0], [-0.3, 0, 0], [0, 0.6, 0]])
    st = R.make_state(pc, rad=[0.2, 0.2, 0.3], mass=[3.0] * 3, inertia=[[0.5, 0.7, 0.9]] * 3, pos_p=pp,
                      clump_id=[0, 0, 0], vel=[[0.1, 0.0, -0.2]] * 3, ang_vel=[[0.0, 0.0, 2.0]] * 3, dtype=f64)
    sy = _sys(3, domain="free", rad=st.rad, dtype=f64, rotation="verletspiral")
    R.free_apply(st, sy)
    assert np.allclose(sy.anchor, np.array([1.0, 2.0, 3.0]) - 0.9) and np.allclose(sy.box_size, 1.8)
    before = R.world_pos(st)
    st, sy = R.step(st, sy, 50)
    after = R.world_pos(st)
    # rigid: pairwise distances of the members are unchanged, the centre drifts at v
    dist = lambda p: np.linalg.norm(p[:, None] - p[None, :], axis=-1)
    assert np.allclose(dist(after), dist(before), atol=1e-9)
    assert np.allclose(st.pos_c[0], [1.0 + 50e-3 * 0.1, 2.0, 3.0 - 50e-3 * 0.2], atol=1e-12)
    assert np.all(st.pos_c == st.pos_c[0]) and np.all(st.ang_vel == st.ang_vel[0])


def test_rigid_clump_wall_impulse_closed_form():
    """ReflectDomain.apply for a clump (reflect.py:165-297): a tilted dumbbell whose lower
    member crosses the wall y = 0 with no force acting (acc = 0, so the contact velocity is
    the end-of-step one): with e = 1 the impulse -(1 + e) v_n / (1/m + (r x n) . I^-1 (r x n))
    reverses the contact point's normal velocity and keeps the kinetic energy (translation
    plus rotation); the clump starts to spin."""
    f64 = np.float64
    th = np.pi / 6
    q = np.array([np.cos(th / 2), 0, 0, np.sin(th / 2)])  # 30 degrees about z
    pp = np.array([[-0.4, 0, 0], [0.4, 0, 0]])
    M, I = 2.0, np.array([0.3, 0.5, 0.6])
    st = R.make_state(np.array([[3.0, 0.49, 3.0]] * 2), rad=[0.3, 0.3], mass=[M] * 2, inertia=[I] * 2,
                      pos_p=pp, clump_id=[0, 0], vel=[[0.2, -1.0, 0.0]] * 2, q=[q] * 2, dtype=f64)
    sy = _sys(3, domain="reflect", box=[10, 10, 10], rad=st.rad, dtype=f64)
    sy.restitution = f64(1.0)
    r = R.pos_p_rot(st)
    ke = lambda s: 0.5 * M * s.vel[0] @ s.vel[0] + 0.5 * (R.quat_rotate_back(s.q, s.ang_vel)[0] ** 2 @ I)
    vc_before = st.vel[0] + np.cross(st.ang_vel[0], r[0])
    e0 = ke(st)
    st2 = R.reflect_apply(st.copy(), sy)
    assert np.isclose(ke(st2), e0, rtol=1e-12)
    # the lower member (index 0, at -0.4 rotated: y = 0.49 - 0.2) took the impulse
    vc_now = st2.vel[0] + np.cross(st2.ang_vel[0], r[0])
    assert np.isclose(vc_now[1], -vc_before[1], rtol=1e-12)
    assert abs(st2.ang_vel[0, 2]) > 0.1 and np.array_equal(st2.ang_vel[0], st2.ang_vel[1])


def test_periodic_image_pair():
    """Minimum image across the boundary (periodic.py:74-79)."""
    L = 10.0
    pos = np.array([[0.2, 5.0, 5.0], [9.6, 5.0, 5.0]], F32)
    rad = np.full(2, 0.5, F32)
    st = R.make_state(pos, rad=rad)
    sy = _sys(3, domain="periodic", box=[L, L, L], rad=rad)
    f, _ = R.cell_list_force(st, sy, sum_dtype=np.float64)
    delta = 1.0 - 0.6
    assert np.allclose(f[0], [1e3 * delta, 0, 0], rtol=1e-5)
    assert np.allclose(f[1], [-1e3 * delta, 0, 0], rtol=1e-5)
    pairs = R.contact_pairs(st, sy)
    assert pairs.tolist() == [[0, 1]]


def test_reflect_wall_bounce_analytic():
    """Free flight into a wall (reflect.py:99-299, _toc.py:11-94): with F = 0 the collision
    fraction is 1 - delta / (|v| dt); the velocity flips and the overshoot is mirrored."""
    v, dt = -2.0, 1e-3
    x0 = 0.5 + 0.0015  # distance to the wall contact point = 1.5e-3 < |v| dt = 2e-3
    pos = np.array([[x0, 5.0]], F32)
    vel = np.array([[v, 0.0]], F32)
    st = R.make_state(pos, vel=vel, rad=np.array([0.5], F32))
    sy = _sys(2, domain="reflect", box=[10, 10], rad=st.rad, dt=dt)
    st, sy = R.step(st, sy, 1)  # drift overshoots the wall by 5e-4
    st = R.reflect_apply(st, sy)  # next step's apply
    assert np.isclose(st.vel[0, 0], -v, rtol=1e-5)
    assert np.isclose(st.pos_c[0, 0], 0.5 + 5e-4, atol=1e-6)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("domain", ["periodic", "reflect", "free"])
@pytest.mark.parametrize("poly", [1.0, 2.0, 3.0])
def test_cell_list_equals_all_pairs(dim, domain, poly):
    """tests/test_colliders_invariance.py:365-402: the cell list sums the same pairs."""
    rng = np.random.default_rng(100 + dim)
    N = 300 if dim == 3 else 200
    rad = rng.uniform(0.5 / poly, 0.5, N).astype(F32)
    L = 7.0 if dim == 3 else 11.0
    pos = rng.uniform(0, L, (N, dim)).astype(F32)
    st = R.make_state(pos, rad=rad)
    sy = _sys(dim, domain=domain, box=np.full(dim, L), rad=rad)
    a, _ = R.cell_list_force(st, sy, sum_dtype=np.float64)
    b = R.naive_force(st, sy, sum_dtype=np.float64)
    assert np.allclose(a, b, rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("domain", ["periodic", "reflect", "free"])
@pytest.mark.parametrize("dim", [2, 3])
def test_c_restatement_matches_numpy_bitwise(domain, dim):
    """The C/OpenMP oracle steps bit-identically to the numpy oracle (float32)."""
    w = W.c1(N=512, seed=5) if dim == 3 else W.c3(N=512, seed=5)
    w.domain = domain
    if domain == "reflect" and dim == 3:
        w.pos = np.clip(w.pos, w.rad[:, None], w.box_size - w.rad[:, None]).astype(F32)
    st = R.make_state(w.pos, vel=w.vel, rad=w.rad, mass=w.mass)
    sy = _sys(dim, domain=domain, box=w.box_size, rad=w.rad, dt=w.dt, gravity=w.gravity)
    st1, sy1 = R.step(st.copy(), sy, 5)
    pos, vel, frc = w.pos.copy(), w.vel.copy(), np.zeros_like(w.pos)
    box, anc = oracle.c_step(dim, pos, vel, frc, w.rad, w.mass, domain=domain, box=w.box_size,
                             anchor=w.anchor, dt=w.dt, steps=5, cell_size=float(sy.cell_size),
                             gravity=w.gravity, threads=2)
    assert np.array_equal(pos, st1.pos_c)
    assert np.array_equal(vel, st1.vel)
    assert np.array_equal(frc, st1.force)
    if domain == "free":
        assert np.array_equal(box, sy1.box_size) and np.array_equal(anc, sy1.anchor)


def _lattice(dim, poly, seed=42):
    """set_up_spheres (tests/test_colliders_invariance.py:50-110): 64 spheres on a
    1.2-spaced lattice, radii U[0.5/poly, 0.5], velocities U[-1, 1], mass 1, k = 1e3."""
    n = int(round(64 ** (1 / dim)))
    axes = [np.arange(n) * 1.2] * dim
    pos = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, dim).astype(np.float64)
    rng = np.random.default_rng(seed)
    rad = rng.uniform(0.5 / poly, 0.5, len(pos))
    vel = rng.uniform(-1, 1, pos.shape)
    return pos, vel, rad, np.full(dim, 1.2 * n), np.full(dim, -0.5)


def _energy_std(dim, domain, linear, dt, total=5.0, n_samples=100, dtype=np.float64):
    """Std of the total energy over a run (the reference runs this under jax_enable_x64)."""
    pos, vel, rad, box, anchor = _lattice(dim, 1.0)
    pos, vel, rad = pos.astype(dtype), vel.astype(dtype), rad.astype(dtype)
    box, anchor = box.astype(dtype), anchor.astype(dtype)
    mass = np.ones(len(pos), dtype)
    frc = np.zeros_like(pos)
    steps = int(total / dt)
    stride = max(1, steps // n_samples)
    cell = 2 * float(rad.max())
    es = []
    st_e = R.make_state(pos, rad=rad, mass=mass, dtype=dtype)
    sy_e = _sys(dim, domain=domain, box=box, anchor=anchor, rad=rad, dtype=dtype)
    for _ in range(n_samples):
        b2, a2 = oracle.c_step(dim, pos, vel, frc, rad, mass, domain=domain, box=box, anchor=anchor, dt=dt,
                               steps=stride, cell_size=cell, linear=linear, threads=1, acc64=True)
        st_e.pos_c, st_e.vel = pos.copy(), vel.copy()
        if domain == "free":
            sy_e.box_size, sy_e.anchor = b2, a2
            sy_e.inv_box_size = (1 / b2).astype(dtype)
        e = R.compute_energy(st_e, sy_e, naive=True)
        es.append(e[0] + e[1] + e[2] + e[3])
    return float(np.std(es))


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("domain", ["periodic", "reflect", "free"])
@pytest.mark.parametrize("linear", ["verlet", "euler"])
def test_energy_conservation_order(dim, domain, linear):
    """tests/test_energy_conservation.py:34-88: slope of log std(E) vs log dt."""
    dts = np.logspace(np.log10(2e-3), np.log10(3e-5), 5)
    stds = [_energy_std(dim, domain, linear, float(dt)) for dt in dts]
    slope, _ = np.polyfit(np.log(dts), np.log(stds), 1)
    if linear == "verlet":
        assert slope > 1.8, (slope, stds)
    else:
        assert slope > 0.7, (slope, stds)


@pytest.mark.parametrize("rot", ["spiral", "verletspiral"])
def test_aspherical_rotation_closed_form(rot):
    """tests/test_rotation_integrators.py:24-97 on the restated integrators (float64):
    constant body-frame torque on an asymmetric body, 70,000 steps of 1e-5."""
    rho, Rad, H = 7750.0, 0.05, 0.15
    M = rho * np.pi * Rad * Rad * H
    Ix = 0.5 * M * Rad * Rad
    Iy = M * H * H / 12.0 + 0.25 * M * Rad * Rad
    Iz = Iy
    tx = Rad * 0.5
    w0 = np.array([0.3, -0.9, 0.6])
    f64 = np.float64
    st = R.make_state(np.zeros((1, 3)), ang_vel=w0[None], mass=np.array([M]), rad=np.array([Rad]), dtype=f64)
    st.inertia = np.array([[Ix, Iy, Iz]], f64)
    sy = _sys(3, domain="free", rad=st.rad, dt=1e-5, rotation=rot, dtype=f64)
    tb = np.array([[tx, 0.0, 0.0]])
    torque_lab = lambda q: R.quat_rotate(q, tb)  # noqa: E731
    st.torque = torque_lab(st.q)
    for _ in range(70000):
        if rot == "verletspiral":
            st = R.vvspiral_before(st, sy)
        st.torque = torque_lab(st.q)  # ForceManager: user torque in the lab frame
        if rot == "verletspiral":
            st = R.vvspiral_after(st, sy)
        else:
            st = R.spiral_after(st, sy)
    t = 0.7
    A = (Ix - Iy) * (Iz - Ix) / (Iy * Iz)
    B = Iy / (Iz - Ix)
    E = 2.0 * tx * B / Ix
    wx = w0[0] + tx * t / Ix
    eta = 0.5 * Ix * np.sqrt(-A) / tx
    C = E * eta
    K1 = (C * w0[1] * np.cos(eta * w0[0] ** 2) - w0[2] * np.sin(eta * w0[0] ** 2)) / C
    K2 = (C * w0[1] * np.sin(eta * w0[0] ** 2) + w0[2] * np.cos(eta * w0[0] ** 2)) / C
    D = eta * wx ** 2
    ww = np.array([wx, K1 * np.cos(D) + K2 * np.sin(D), C * (K2 * np.cos(D) - K1 * np.sin(D))])
    wb = R.quat_rotate_back(st.q, st.ang_vel)[0]
    assert np.log10(np.linalg.norm(wb - ww) / np.linalg.norm(ww)) < -4.0


@pytest.mark.parametrize("cfg,cell,grid", [("c1", 1.0, (17, 17, 17)), ("c2", 1.4, (87, 87, 87)),
                                           ("c3", 1.2, (1820, 1820))])
def test_grid_parameters_of_the_configurations(cfg, cell, grid):
    """DynamicCellList.Create + _grid_params (cell_list.py:374-432, _partition.py:54-99)."""
    w = {"c1": lambda: W.c1(), "c2": lambda: W.c2(N=4096), "c3": lambda: W.c3(N=4096)}[cfg]()
    if cfg == "c2":  # box of the full-size system
        w.box_size = np.full(3, 123.17252, F32)
    if cfg == "c3":
        w.box_size = np.full(2, 2183.75, F32)
    c, mask = R.cell_list_create(w.rad if cfg != "c3" else np.array([0.4, 0.6], F32), w.dim)
    assert np.isclose(c, cell, rtol=1e-6)
    assert mask.shape == (3 ** w.dim, w.dim)
    g, strides, _, ovf = R.grid_params(w.box_size, c, w.domain == "periodic")
    assert tuple(g) == grid and not ovf


def test_neighbor_list_properties():
    """create_neighbor_list rows: within the cutoff, symmetric, no self, -1 padded."""
    w = W.c1(N=600, seed=9)
    st = R.make_state(w.pos, rad=w.rad)
    sy = _sys(3, domain="periodic", box=w.box_size, rad=w.rad)
    nl, ovf = R.create_neighbor_list(st, sy, 1.5, 40)
    assert not ovf
    rows = [set(r[r >= 0].tolist()) for r in nl]
    for i, r in enumerate(rows):
        assert i not in r
        for j in r:
            assert i in rows[j]
            d = R.displacement_true(w.pos[i], w.pos[j], sy)
            assert float(np.sum(d.astype(np.float64) ** 2)) <= 1.5 ** 2 * (1 + 1e-6)
