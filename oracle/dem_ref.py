"""CPU restatement of JaxDEM's per-step hot path, in numpy.

TEST INFRASTRUCTURE ONLY.  This module is the oracle (the checker): only
``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` may import it.  The product path (``jaxdem_gb300``) never
touches it; there is no CPU fallback.

Every function restates the reference algorithm with the same float32
operation order as the cited JAX code, so that pair terms, contact sets and
integrator updates agree bit for bit with the CUDA kernels (which are built
without FMA contraction).  Paths below are relative to the JaxDEM project.

Parity pinning.  JAX is not importable in this environment, so the oracle
cannot be compared against the reference's own outputs.  The reference ships
no stored golden arrays; it is pinned instead against the reference's own
known-answer tests restated in ``tests/test_oracle_pins.py``:
``tests/test_excluded_pairs.py:11-61`` (bond exclusion, F0 = -F2),
``tests/test_energy_conservation.py:34-107`` (Verlet energy-error slope
> 1.8), ``tests/test_colliders_invariance.py:365-402`` (cell list equals
naive all-pairs), ``tests/test_rotation_integrators.py`` (analytic
rigid-body rotation) and hand-derived analytic answers (two-sphere spring,
periodic image pair, single-sphere wall reflection).  Bit-level parity with
XLA itself (summation order inside ``jnp.sum``) is unpinned.

Summation order.  The reference folds each particle's candidates per
stencil cell in chunks of ``PAIR_UNROLL = 4`` (``colliders/cell_list.py:
184,235-254``) and then sums the stencil cells
(``colliders/cell_list.py:257-258``).  XLA's internal order for those
reductions is not specified; this restatement sums left to right.
"""

from __future__ import annotations

from dataclasses import dataclass, field, replace
from typing import Optional

import numpy as np

PAIR_UNROLL = 4  # colliders/cell_list.py:184


# ---------------------------------------------------------------------------
# Containers.  Plain numpy arrays in the reference's (N, dim) layout.
# ---------------------------------------------------------------------------


@dataclass
class OState:
    """Particle record, fields as ``State`` (``state.py:103-228``): spheres, or rigid
    clumps whose members store the clump's pos_c, vel, q, ang_vel, mass and inertia."""

    pos_c: np.ndarray  # (N, d)
    vel: np.ndarray  # (N, d)
    force: np.ndarray  # (N, d)
    q: np.ndarray  # (N, 4) w, x, y, z
    ang_vel: np.ndarray  # (N, 1|3)
    torque: np.ndarray  # (N, 1|3)
    rad: np.ndarray  # (N,)
    mass: np.ndarray  # (N,)
    inertia: np.ndarray  # (N, 1|3)
    mat_id: np.ndarray  # (N,) int
    fixed: np.ndarray  # (N,) bool
    bond_id: np.ndarray  # (N, W) int, -1 padded
    clump_id: np.ndarray  # (N,) int
    pos_p: Optional[np.ndarray] = None  # (N, d) body-frame offsets of rigid-clump members

    @property
    def N(self) -> int:
        return self.pos_c.shape[0]

    @property
    def dim(self) -> int:
        return self.pos_c.shape[1]

    def copy(self) -> "OState":
        return OState(**{k: None if v is None else np.array(v, copy=True) for k, v in self.__dict__.items()})

    @property
    def rigid(self) -> bool:
        """Rigid clumps present (an offset, or a clump id shared by several spheres)."""
        if self.pos_p is not None and np.any(self.pos_p != 0):
            return True
        return bool(np.any(self.clump_id != np.arange(self.N)))


@dataclass
class OSystem:
    """Configuration scalars of ``System`` (``system.py:160-226``) for the hot path."""

    dim: int
    domain: str  # "periodic" | "reflect" | "free"
    box_size: np.ndarray
    anchor: np.ndarray
    young_eff: np.ndarray  # (M, M): spring k, or (4/3) E* when force_law == "hertz"
    dt: np.floating
    cell_size: np.floating
    neighbor_mask: np.ndarray  # (M_st, d) int
    gravity: np.ndarray
    restitution: np.floating = np.float32(1.0)
    linear: str = "verlet"
    rotation: str = "verletspiral"
    interact_same_bond_id: bool = False
    time: np.floating = np.float32(0.0)
    step_count: int = 0
    inv_box_size: Optional[np.ndarray] = None
    force_law: str = "spring"  # "spring" | "hertz" | "cundallstrack" (forces/*.py)
    mat_props: Optional[np.ndarray] = None  # cundallstrack: (M, 4) young, shear modulus, mu, mu_r
    # NeighborList collider (colliders/neighbor_list.py): cutoff, skin, max_neighbors and the
    # cached list, reference positions and build count; None for the cell list
    nlist: Optional[dict] = None

    def __post_init__(self) -> None:
        if self.inv_box_size is None:
            self.inv_box_size = (1.0 / self.box_size).astype(self.box_size.dtype)

    @property
    def periodic(self) -> bool:
        return self.domain == "periodic"


def make_state(pos, vel=None, rad=None, mass=None, density=None, mat_id=None,
               fixed=None, bond_id=None, ang_vel=None, torque=None, q=None,
               force=None, dtype=np.float32, pos_p=None, clump_id=None, inertia=None) -> OState:
    """Defaults of ``State.create`` (``state.py:640-862``) for spheres."""
    pos = np.asarray(pos, dtype)
    N, d = pos.shape
    ad = 1 if d == 2 else 3
    rad = np.ones(N, dtype) if rad is None else np.asarray(rad, dtype)
    mat_id = np.zeros(N, np.int32) if mat_id is None else np.asarray(mat_id, np.int32)
    if density is not None:
        # mass = density[mat_id] * volume  (state.py:807-809)
        vol = hypersphere_volume(rad, d, dtype)
        mass = np.asarray(density, dtype)[mat_id] * vol
    mass = np.ones(N, dtype) if mass is None else np.asarray(mass, dtype)
    ang_vel = np.zeros((N, ad), dtype) if ang_vel is None else np.asarray(ang_vel, dtype).reshape(N, ad)
    coeff = dtype(0.5) if d == 2 else dtype(0.4)
    if inertia is None:
        inertia = ((coeff * mass) * rad * rad)[:, None] * np.ones((N, ad), dtype)  # state.py:817-823
    else:
        inertia = np.asarray(inertia, dtype).reshape(N, ad).copy()
    if q is None:
        q = np.zeros((N, 4), dtype)
        q[:, 0] = 1
    return OState(
        pos_c=pos.copy(),
        vel=np.zeros((N, d), dtype) if vel is None else np.asarray(vel, dtype).copy(),
        force=np.zeros((N, d), dtype) if force is None else np.asarray(force, dtype).copy(),
        q=np.asarray(q, dtype).copy(),
        ang_vel=ang_vel.copy(),
        torque=np.zeros((N, ad), dtype) if torque is None else np.asarray(torque, dtype).reshape(N, ad).copy(),
        rad=rad.copy(),
        mass=mass.copy(),
        inertia=inertia,
        mat_id=mat_id,
        fixed=np.zeros(N, bool) if fixed is None else np.asarray(fixed, bool),
        bond_id=np.full((N, 1), -1, np.int64) if bond_id is None else np.asarray(bond_id, np.int64),
        clump_id=np.arange(N, dtype=np.int64) if clump_id is None else np.asarray(clump_id, np.int64),
        pos_p=np.zeros((N, d), dtype) if pos_p is None else np.asarray(pos_p, dtype).copy(),
    )


def hypersphere_volume(rad, dim, dtype=np.float32):
    """Sphere volume / disk area used by ``State.create`` for the default mass."""
    rad = np.asarray(rad, dtype)
    if dim == 2:
        return dtype(np.pi) * rad * rad
    return (dtype(4.0 / 3.0) * dtype(np.pi)) * rad * rad * rad


# ---------------------------------------------------------------------------
# Cell-list parameters and partition.
# ---------------------------------------------------------------------------


def cell_list_create(rad, dim, cell_size=None, search_range=None, box_size=None,
                     dtype=np.float32):
    """``DynamicCellList.Create`` (``colliders/cell_list.py:374-432``).

    Returns ``(cell_size, neighbor_mask)``; the mask lists the integer offsets
    of ``meshgrid(indexing="ij")`` raveled, i.e. the last axis varies fastest.
    """
    rad = np.asarray(rad, dtype)
    min_rad = rad.min()
    max_rad = rad.max()
    alpha = max_rad / min_rad
    if cell_size is None:
        cell_size = dtype(2.0) * max_rad if alpha < 2.5 else dtype(0.5) * max_rad
    cell_size = dtype(cell_size)
    if box_size is not None:
        box_size = np.asarray(box_size, dtype)
        for _ in range(2):
            if search_range is None:
                sr = max(1, int(np.ceil(dtype(2) * max_rad / cell_size)))
            else:
                sr = int(search_range)
            min_grids = 2 * sr + 1
            g = np.maximum(np.floor(box_size / cell_size).astype(np.int64), min_grids)
            cell_size = np.min(box_size / g.astype(dtype)).astype(dtype)
    if search_range is None:
        search_range = max(1, int(np.ceil(dtype(2) * max_rad / cell_size)))
    r = np.arange(-search_range, search_range + 1)
    mesh = np.meshgrid(*([r] * dim), indexing="ij")
    neighbor_mask = np.stack([m.ravel() for m in mesh], axis=1).astype(np.int64)
    return dtype(cell_size), neighbor_mask


def grid_params(box_size, cell_size, periodic):
    """``_grid_params`` (``colliders/_partition.py:54-99``)."""
    box_size = np.asarray(box_size)
    dt = box_size.dtype
    if periodic:
        g = np.maximum(np.floor(box_size / cell_size).astype(np.int64), 1)
        cell = (box_size / g.astype(dt)).astype(dt)
    else:
        g = np.maximum(np.ceil(box_size / cell_size).astype(np.int64), 1)
        cell = np.full_like(box_size, cell_size)
    strides = np.concatenate([[1], np.cumprod(g[:-1])]).astype(np.int64)
    overflow = float(np.prod(g.astype(np.float64))) > float(np.iinfo(np.int32).max)
    return g, strides, cell, overflow


def _floor_mod1(x):
    """``jnp.remainder(x, 1)`` (floor modulo) in the array's dtype."""
    m = np.fmod(x, x.dtype.type(1))
    m = np.where(m < 0, m + x.dtype.type(1), m)
    return m


def cell_coords(pos, sy: OSystem, cell_size):
    """Cell coordinates of ``_get_spatial_partition`` (``cell_list.py:55-60``).

    Coordinates are clamped into ``[0, grid)``.  The reference leaves them
    unclamped, which only differs when ``(pos-anchor)/box mod 1`` rounds up
    to 1.0 or a non-periodic particle lies outside the box; there the
    reference aliases the particle into another cell.  The clamped form is the
    physically correct cell and is what the CUDA binning computes.
    """
    g, strides, cell, _ = grid_params(sy.box_size, cell_size, sy.periodic)
    if sy.periodic:
        frac = _floor_mod1((pos - sy.anchor) / sy.box_size)
        c = np.floor(frac * g.astype(pos.dtype)).astype(np.int64)
    else:
        c = np.floor((pos - sy.anchor) / cell_size).astype(np.int64)
    c = np.clip(c, 0, g - 1)
    return c, g, strides


def spatial_partition(pos, sy: OSystem, cell_size, neighbor_mask):
    """``_get_spatial_partition`` (``colliders/cell_list.py:35-87``).

    Stable sort of ``(hash, iota)`` (``cell_list.py:64``), stencil hashes with
    periodic floor-mod wrap or -1 for out-of-grid cells (``:66-80``).
    """
    c, g, strides = cell_coords(pos, sy, cell_size)
    h = c @ strides
    perm = np.argsort(h, kind="stable")
    sorted_h = h[perm]
    nc = c[:, None, :] + neighbor_mask[None, :, :]
    if sy.periodic:
        nc = nc - g * np.floor_divide(nc, g)
        nh = nc @ strides
    else:
        oob = np.any((nc < 0) | (nc >= g), axis=-1)
        nh = np.where(oob, -1, nc @ strides)
    return perm, sorted_h, nh


def dedup_stencil_exact(nh_orig):
    """``_dedup_stencil_hashes`` (``cell_list.py:90-96``), row-wise.

    Entry ``b`` becomes -1 when an earlier entry of the original row holds
    the same hash (the ``triu(k=1)`` mask reduced over axis 0).
    """
    out = nh_orig.copy()
    M = nh_orig.shape[1]
    for a in range(M):
        dup = np.zeros(nh_orig.shape[0], bool)
        for b in range(a):
            dup |= nh_orig[:, b] == nh_orig[:, a]
        out[:, a] = np.where(dup, -1, nh_orig[:, a])
    return out


# ---------------------------------------------------------------------------
# Pair kernel.
# ---------------------------------------------------------------------------


def displacement_fast(ri, rj, sy: OSystem):
    """``Domain._displacement`` (``domains/periodic.py:74-79``, base ``__init__.py:153-154``)."""
    rij = ri - rj
    if sy.periodic:
        rij = rij - sy.box_size * np.round(rij * sy.inv_box_size)
    return rij


def displacement_true(ri, rj, sy: OSystem):
    """``PeriodicDomain.displacement`` (``domains/periodic.py:37-71``): divides by the box."""
    rij = ri - rj
    if sy.periodic:
        rij = rij - sy.box_size * np.round(rij / sy.box_size)
    return rij


def sumsq(v):
    """Left-to-right ``sum(v**2, axis=-1)``."""
    acc = v[..., 0] * v[..., 0]
    for a in range(1, v.shape[-1]):
        acc = acc + v[..., a] * v[..., a]
    return acc


def spring_pair(i, j, pos, rad, mat_id, young_eff, sy: OSystem):
    """``SpringForce.force`` (``forces/spring.py:69-108``), vectorised over pairs.

    Returns the force on ``i`` due to ``j``; torque is identically zero.
    """
    dt = pos.dtype.type
    R = rad[i] + rad[j]
    rij = displacement_fast(pos[i], pos[j], sy)
    d_sq = sumsq(rij)
    k = young_eff[mat_id[i], mat_id[j]]
    safe = np.maximum(d_sq, dt(1e-16))
    with np.errstate(divide="ignore"):
        inv = np.where(d_sq == 0, dt(0), dt(1) / np.sqrt(safe))
    r = d_sq * inv
    delta = np.maximum(dt(0), R - r) * (np.asarray(i) != np.asarray(j)).astype(pos.dtype)
    mag = k * delta * inv
    return mag[..., None] * rij


def spring_energy_pair(i, j, pos, rad, mat_id, young_eff, sy: OSystem):
    """``SpringForce.energy`` (``forces/spring.py:110-147``)."""
    dt = pos.dtype.type
    R = rad[i] + rad[j]
    rij = displacement_fast(pos[i], pos[j], sy)
    d_sq = sumsq(rij)
    k = young_eff[mat_id[i], mat_id[j]]
    safe = np.maximum(d_sq, dt(1e-16))
    with np.errstate(divide="ignore"):
        inv = np.where(d_sq == 0, dt(0), dt(1) / np.sqrt(safe))
    r = d_sq * inv
    s = np.maximum(dt(0), R - r) * (np.asarray(i) != np.asarray(j)).astype(pos.dtype)
    return dt(0.5) * k * s * s


def hertz_constant(young, poisson):
    """(M, M) table (4/3) E* of ``HertzianForce`` (``forces/hertz.py:99-105``), float32:
    E* = 1 / ((1 - nu_i**2) / E_i + (1 - nu_j**2) / E_j)."""
    E = np.asarray(young, np.float32).reshape(-1)
    nu = np.asarray(poisson, np.float32).reshape(-1)
    a = (np.float32(1.0) - nu ** 2) / E
    return (np.float32(4.0 / 3.0) * (np.float32(1.0) / (a[:, None] + a[None, :]))).astype(np.float32)


def hertz_pair(i, j, pos, rad, mat_id, k43, sy: OSystem):
    """``HertzianForce.force`` (``forces/hertz.py:63-117``), vectorised over pairs:
    k = (4/3) E* sqrt(R*), R* = Ri Rj / (Ri + Rj); F = k pow(delta, 1.5) n with
    (n, r) = unit_and_norm(r_ij) (``utils/linalg.py:164-181``)."""
    dt = pos.dtype.type
    Ri, Rj = rad[i], rad[j]
    R_star = (Ri * Rj) / (Ri + Rj)
    k = k43[mat_id[i], mat_id[j]] * np.sqrt(R_star)
    rij = displacement_fast(pos[i], pos[j], sy)
    n2 = sumsq(rij)
    safe = np.maximum(n2, dt(1e-16))
    with np.errstate(divide="ignore"):
        inv = np.where(n2 == 0, dt(0), dt(1) / np.sqrt(safe))
    r = n2 * inv
    n = rij * inv[..., None]
    delta = np.maximum(dt(0), Ri + Rj - r) * (np.asarray(i) != np.asarray(j)).astype(pos.dtype)
    mag = k * np.power(delta, dt(1.5))
    return mag[..., None] * n


def hertz_energy_pair(i, j, pos, rad, mat_id, k43, sy: OSystem):
    """``HertzianForce.energy`` (``forces/hertz.py:119-160``): 0.4 k pow(delta, 2.5)
    with r = norm(r_ij) (``utils/linalg.py:115-133``)."""
    dt = pos.dtype.type
    Ri, Rj = rad[i], rad[j]
    R_star = (Ri * Rj) / (Ri + Rj)
    k = k43[mat_id[i], mat_id[j]] * np.sqrt(R_star)
    rij = displacement_fast(pos[i], pos[j], sy)
    n2 = sumsq(rij)
    r = np.where(n2 == 0, dt(0), np.sqrt(np.maximum(n2, dt(1e-16))))
    delta = Ri + Rj - r
    delta = delta * (delta > 0).astype(pos.dtype) * (np.asarray(i) != np.asarray(j)).astype(pos.dtype)
    return dt(0.4) * k * np.power(delta, dt(2.5))


def cs_tables(young, poisson, e, mu, mu_r):
    """``CundallStrackForce`` material terms (``forces/cundall_strack.py:128-150``):
    the damping ratio beta (M, M) of e_eff = min(e_i, e_j) (1 where e_eff = 0) and
    per material (young, G = E / (2 (1 + nu)), mu, mu_r) (M, 4), float32."""
    f = np.float32
    E = np.asarray(young, f).reshape(-1)
    nu = np.asarray(poisson, f).reshape(-1)
    G = E / (f(2.0) * (f(1.0) + nu))
    ev = np.asarray(e, f).reshape(-1)
    e_eff = np.minimum(ev[:, None], ev[None, :])
    ln_e = np.log(np.where(e_eff > 0, e_eff, f(1.0))).astype(f)
    beta = np.where(e_eff > 0, -ln_e / np.sqrt(f(np.pi ** 2) + ln_e ** 2), f(1.0)).astype(f)
    props = np.stack([E, G, np.asarray(mu, f).reshape(-1), np.asarray(mu_r, f).reshape(-1)], 1).astype(f)
    return beta, props


def _unit_and_norm(v):
    """``unit_and_norm`` (``utils/linalg.py:164-181``)."""
    dt = v.dtype.type
    n2 = sumsq(v)
    with np.errstate(divide="ignore"):
        inv = np.where(n2 == 0, dt(0), dt(1) / np.sqrt(np.maximum(n2, dt(1e-16))))
    return v * inv[..., None], n2 * inv


def _cross_w(w, r):
    """``cross_3X3D_1X2D(w, r)`` (``utils/linalg.py:184-230``): w x r, 2D w = (0, 0, w_z)."""
    if r.shape[-1] == 3:
        return cross3(w, r)
    return np.concatenate([-w * r[..., 1:2], w * r[..., 0:1]], axis=-1)


def cs_pair(i, j, st, sy: OSystem):
    """``CundallStrackForce.force`` (``forces/cundall_strack.py:100-196``), vectorised over
    pairs: the force on ``i`` due to ``j`` and the torque on ``i``, concatenated
    ``(..., dim + ang_dim)``.  Positions are ``state.pos`` (members' world positions for
    clumps); velocities, spins and masses are the members' stored (clump) values."""
    pos = world_pos(st)
    dt = pos.dtype.type
    d = pos.shape[-1]
    mi, mj = st.mat_id[i], st.mat_id[j]
    P = sy.mat_props.astype(pos.dtype)
    E_i, E_j, G_i, G_j = P[mi, 0], P[mj, 0], P[mi, 1], P[mj, 1]
    R_i, R_j = st.rad[i], st.rad[j]
    m_i, m_j = st.mass[i], st.mass[j]
    kn = (dt(2.0) * E_i * R_i * E_j * R_j) / (E_i * R_i + E_j * R_j)
    kt = (dt(2.0) * G_i * R_i * G_j * R_j) / (G_i * R_i + G_j * R_j)
    m_eff = (m_i * m_j) / (m_i + m_j)
    mu_eff = np.minimum(P[mi, 2], P[mj, 2])
    beta = sy.young_eff.astype(pos.dtype)[mi, mj]
    gamma_n = dt(2.0) * beta * np.sqrt(kn * m_eff)
    gamma_t = dt(2.0) * beta * np.sqrt(kt * m_eff)
    rij = displacement_fast(pos[i], pos[j], sy)
    n, r = _unit_and_norm(rij)
    delta = R_i + R_j - r
    contact = ((delta > 0) & (np.asarray(i) != np.asarray(j))).astype(pos.dtype)
    delta = delta * contact
    r_ci = -R_i[..., None] * n
    r_cj = R_j[..., None] * n
    w = st.ang_vel
    v_ci = st.vel[i] + _cross_w(w[i], r_ci)
    v_cj = st.vel[j] + _cross_w(w[j], r_cj)
    v_rel = v_ci - v_cj
    vn = sumsq_dot(v_rel, n)
    t, vt = _unit_and_norm(v_rel - vn[..., None] * n)
    Fn = np.maximum(dt(0), kn * delta - gamma_n * vn) * contact
    Ft = np.minimum(gamma_t * vt, mu_eff * Fn) * contact
    F = Fn[..., None] * n - Ft[..., None] * t
    if d == 3:
        tq = cross3(r_ci, F)
    else:
        tq = r_ci[..., 0:1] * F[..., 1:2] - r_ci[..., 1:2] * F[..., 0:1]
    mu_r = np.minimum(P[mi, 3], P[mj, 3])
    R_eff = (R_i * R_j) / (R_i + R_j)
    w_rel = w[i] - w[j]
    n2 = sumsq(w_rel)
    w_hat = w_rel * (dt(1) / np.sqrt(np.where(n2 == 0, dt(1), n2)))[..., None]
    tq = tq - (mu_r * R_eff * Fn)[..., None] * w_hat
    return np.concatenate([F, tq], axis=-1)


def sumsq_dot(a, b):
    """Left-to-right dot product along the last axis."""
    acc = a[..., 0] * b[..., 0]
    for k in range(1, a.shape[-1]):
        acc = acc + a[..., k] * b[..., k]
    return acc


def cs_energy_pair(i, j, pos, rad, mat_id, sy: OSystem):
    """``CundallStrackForce.energy`` (``forces/cundall_strack.py:197-236``): 0.5 kn delta^2."""
    dt = pos.dtype.type
    P = sy.mat_props.astype(pos.dtype)
    E_i, E_j = P[mat_id[i], 0], P[mat_id[j], 0]
    R_i, R_j = rad[i], rad[j]
    kn = (dt(2.0) * E_i * R_i * E_j * R_j) / (E_i * R_i + E_j * R_j)
    rij = displacement_fast(pos[i], pos[j], sy)
    n2 = sumsq(rij)
    r = np.where(n2 == 0, dt(0), np.sqrt(np.maximum(n2, dt(1e-16))))
    delta = R_i + R_j - r
    delta = delta * (delta > 0).astype(pos.dtype) * (np.asarray(i) != np.asarray(j)).astype(pos.dtype)
    return dt(0.5) * kn * delta * delta


def pair_force(i, j, pos, rad, mat_id, sy: OSystem):
    """The force law of ``sy`` (``System.force_model.force``)."""
    if sy.force_law == "hertz":
        return hertz_pair(i, j, pos, rad, mat_id, sy.young_eff, sy)
    return spring_pair(i, j, pos, rad, mat_id, sy.young_eff, sy)


def pair_energy(i, j, pos, rad, mat_id, sy: OSystem):
    """The force law's pair energy (``System.force_model.energy``)."""
    if sy.force_law == "cundallstrack":
        return cs_energy_pair(i, j, pos, rad, mat_id, sy)
    if sy.force_law == "hertz":
        return hertz_energy_pair(i, j, pos, rad, mat_id, sy.young_eff, sy)
    return spring_energy_pair(i, j, pos, rad, mat_id, sy.young_eff, sy)


def valid_mask(clump_i, clump_j, bond_row_i, index_j, interact_same_bond_id):
    """``valid_interaction_mask`` (``colliders/__init__.py:225-243``)."""
    is_bonded = np.any(bond_row_i == np.asarray(index_j)[..., None], axis=-1)
    return (clump_i != clump_j) & ((~is_bonded) | bool(interact_same_bond_id))


def pos_p_rot(st: OState):
    """``state._pos_p_rot`` (``state.py:230-273``): R(q) pos_p, zero for spheres."""
    if st.pos_p is None or not np.any(st.pos_p != 0):
        return np.zeros_like(st.pos_c)
    return quat_rotate(st.q, st.pos_p).astype(st.pos_c.dtype)


def world_pos(st: OState):
    """``State.pos`` (``state.py:295-304``): pos_c + R(q) pos_p."""
    if st.pos_p is None or not np.any(st.pos_p != 0):
        return st.pos_c
    return st.pos_c + pos_p_rot(st)


def _traverse(st: OState, sy: OSystem, pair_fn, acc_shape, acc_dtype, sum_dtype=None):
    """``_traverse_pairs`` (``colliders/cell_list.py:187-261``), vectorised over particles.

    ``sum_dtype`` selects the accumulator precision (float32 reproduces the
    reference's accumulation; float64 gives the exactly rounded sum of the
    float32 pair terms, used as the tighter force check).
    """
    N = st.N
    pos = world_pos(st)
    sum_dtype = acc_dtype if sum_dtype is None else sum_dtype
    perm, sorted_h, nh = spatial_partition(pos, sy, sy.cell_size, sy.neighbor_mask)
    if sy.periodic:
        nh = dedup_stencil_exact(nh)
    iota = np.arange(N)
    total = np.zeros((N,) + acc_shape, sum_dtype)
    for m in range(nh.shape[1]):
        target = nh[:, m]
        start = np.searchsorted(sorted_h, target, side="left")
        acc = np.zeros((N,) + acc_shape, sum_dtype)
        k = start.copy()
        active = (k < N) & (sorted_h[np.minimum(k, N - 1)] == target) & (target != -1)
        while active.any():
            idx = np.nonzero(active)[0]
            chunk = np.zeros((idx.size,) + acc_shape, sum_dtype)
            for u in range(PAIR_UNROLL):
                ku = k[idx] + u
                kj = np.minimum(ku, N - 1)
                in_cell = (ku < N) & (sorted_h[kj] == target[idx])
                j = perm[kj]
                ok = in_cell & valid_mask(st.clump_id[j], st.clump_id[idx], st.bond_id[j],
                                          idx, sy.interact_same_bond_id)
                v = pair_fn(idx, j).astype(sum_dtype)
                mask = ok.reshape((-1,) + (1,) * len(acc_shape))
                chunk = chunk + np.where(mask, v, 0)
            acc[idx] = acc[idx] + chunk
            k[idx] += PAIR_UNROLL
            kk = np.minimum(k, N - 1)
            active = active & (k < N) & (sorted_h[kk] == target)
        total = total + acc
    return total


def cell_list_force(st: OState, sy: OSystem, sum_dtype=None):
    """``DynamicCellList.compute_force`` (``colliders/cell_list.py:434-464``).

    Returns ``(force, torque)`` with torque = sum of pair torques + cross(R(q) pos_p, F):
    ``0 + cross(0, F) = 0`` for smooth spheres.
    """
    pos = world_pos(st)
    d = st.dim
    if sy.force_law == "cundallstrack":
        # force and torque summed together; torque + cross(R(q) pos_p, F) (cell_list.py:452-464)
        ad = st.torque.shape[-1]
        ft = _traverse(st, sy, lambda i, j: cs_pair(i, j, st, sy), (d + ad,), pos.dtype, sum_dtype)
        f, tq = ft[:, :d].astype(pos.dtype), ft[:, d:].astype(pos.dtype)
        if st.rigid:
            r = pos_p_rot(st)
            tq = tq + (cross3(r, f) if d == 3 else r[:, 0:1] * f[:, 1:2] - r[:, 1:2] * f[:, 0:1])
        return f, tq.astype(pos.dtype)

    def pair(i, j):
        return pair_force(i, j, pos, st.rad, st.mat_id, sy)

    f = _traverse(st, sy, pair, (d,), pos.dtype, sum_dtype).astype(pos.dtype)
    if not st.rigid:
        return f, np.zeros_like(st.torque)
    r = pos_p_rot(st)
    t = pos.dtype.type
    if d == 3:
        tq = t(0) + cross3(r, f)
    else:
        tq = t(0) + (r[:, 0:1] * f[:, 1:2] - r[:, 1:2] * f[:, 0:1])
    return f, tq.astype(pos.dtype)


def neighbor_list_collider(cutoff, skin, max_neighbors, dtype=np.float32):
    """A NeighborList collider's cache before its first build (``neighbor_list.py:287-420``)."""
    return {"cutoff": dtype(cutoff), "skin": dtype(skin), "max": int(max_neighbors), "nl": None, "old_pos": None,
            "builds": 0}


def neighbor_list_force(st: OState, sy: OSystem):
    """``NeighborList.compute_force`` (``colliders/neighbor_list.py:594-661``).

    ``_check_and_rebuild`` (``:58-130``): the list is rebuilt when the largest unwrapped
    displacement since the last build exceeds skin / 2 (squared: skin**2 / 4) or before the
    first build, by the cell list's ``create_neighbor_list`` at cutoff + skin (``_rebuild``,
    ``:545-592``).  Each particle then sums its row in list order, padding and excluded
    entries as zero terms (``jnp.sum`` over the row), and adds cross(R(q) pos_p, F) to the
    torque sum.  Updates the cache in ``sy.nlist``; returns ``(force, torque)``.
    """
    c = sy.nlist
    pos = world_pos(st)
    dt = pos.dtype.type
    rebuild = c["builds"] == 0
    if not rebuild:
        disp = pos - c["old_pos"]
        rebuild = bool(np.max(sumsq(disp)) > c["skin"] ** 2 / dt(4))
    if rebuild:
        c["nl"], _ = create_neighbor_list(st, sy, dt(c["cutoff"] + c["skin"]), c["max"])
        c["old_pos"] = pos.copy()
        c["builds"] += 1
    nl = c["nl"]
    N, d = pos.shape
    ad = st.torque.shape[-1]
    f = np.zeros((N, d), pos.dtype)
    tq = np.zeros((N, ad), pos.dtype)
    iota = np.arange(N)
    for m in range(nl.shape[1]):
        j = nl[:, m]
        safe = np.maximum(j, 0)
        valid = (j != -1) & valid_mask(st.clump_id[iota], st.clump_id[safe], st.bond_id, safe,
                                       sy.interact_same_bond_id)
        if sy.force_law == "cundallstrack":
            ft = cs_pair(iota, safe, st, sy)
            fi, ti = ft[:, :d], ft[:, d:]
        else:
            fi, ti = pair_force(iota, safe, pos, st.rad, st.mat_id, sy), np.zeros((N, ad), pos.dtype)
        fi = np.where(valid[:, None], fi, dt(0))
        ti = np.where(valid[:, None], ti, dt(0))
        # jnp.sum over the row: the first entry, then left to right
        f = fi if m == 0 else f + fi
        tq = ti if m == 0 else tq + ti
    r = pos_p_rot(st)
    tq = tq + (cross3(r, f) if d == 3 else r[:, 0:1] * f[:, 1:2] - r[:, 1:2] * f[:, 0:1])
    return f.astype(pos.dtype), tq.astype(pos.dtype)


def collider_force(st: OState, sy: OSystem, sum_dtype=None):
    """``system.collider.compute_force``: the NeighborList collider when ``sy.nlist`` is set,
    else the cell list."""
    if sy.nlist is not None:
        return neighbor_list_force(st, sy)
    return cell_list_force(st, sy, sum_dtype)


def cell_list_energy(st: OState, sy: OSystem, sum_dtype=None):
    """``DynamicCellList.compute_potential_energy`` (``cell_list.py:466-496``), pair term x0.5 (``_partition.py:39-51``)."""
    pos = world_pos(st)
    half = pos.dtype.type(0.5)

    def pair(i, j):
        return half * pair_energy(i, j, pos, st.rad, st.mat_id, sy)

    e = _traverse(st, sy, pair, (), pos.dtype, sum_dtype)
    return e.sum(dtype=np.float64)


def naive_force(st: OState, sy: OSystem, sum_dtype=np.float64):
    """``NaiveSimulator.compute_force`` (``colliders/naive.py:187-235``), O(N^2)."""
    N = st.N
    pos = world_pos(st)
    iota = np.arange(N)
    out = np.zeros((N, st.dim), sum_dtype)
    for i in range(N):
        f = pair_force(np.full(N, i), iota, pos, st.rad, st.mat_id, sy)
        ok = valid_mask(st.clump_id[i], st.clump_id, st.bond_id[i][None, :], iota,
                        sy.interact_same_bond_id)
        out[i] = np.where(ok[:, None], f, 0).astype(sum_dtype).sum(axis=0)
    return out.astype(pos.dtype)


# ---------------------------------------------------------------------------
# Domains, force manager, integrators.
# ---------------------------------------------------------------------------


def verlet_collision_fraction(v_end, acc, delta, wall_sign, dt):
    """``verlet_collision_fraction`` (``domains/_toc.py:11-94``)."""
    t = v_end.dtype.type
    v_0 = v_end - dt * acc
    v_mid = v_end - t(0.5) * dt * acc
    v_0_n = v_0 * wall_sign
    v_mid_n = v_mid * wall_sign
    acc_n = acc * wall_sign
    A = t(0.5) * acc_n * dt * dt
    B = v_0_n * dt
    d_wall = delta + v_mid_n * dt
    disc = B * B + t(4.0) * A * d_wall
    disc = np.maximum(t(0), disc)
    safe = np.where(disc > 0, disc, t(1))
    sq = np.where(disc > 0, np.sqrt(safe), t(0))
    with np.errstate(divide="ignore", invalid="ignore"):
        den1 = np.where(B - sq < t(-1e-10), B - sq, t(-1.0))
        den2 = np.where(np.abs(t(2.0) * A) > t(1e-10), t(2.0) * A, t(1.0))
        alpha = np.where(B < 0, t(2.0) * d_wall / den1, (-B - sq) / den2)
    return np.clip(alpha, t(0), t(1))


def reflect_apply(st: OState, sy: OSystem):
    """``ReflectDomain.apply`` (``domains/reflect.py:99-299``) for spheres.

    With ``clump_id == iota`` and ``pos_p == 0`` every segment reduction is
    the identity, the rotational denominator and lever-arm terms vanish and
    ``count_active`` equals ``active``.
    """
    if st.rigid:
        return reflect_apply_clumps(st, sy)
    t = st.pos_c.dtype.type
    e = t(sy.restitution)
    pos = st.pos_c
    rad = st.rad[:, None]
    lo = sy.anchor + rad
    hi = sy.anchor + sy.box_size - rad
    over_lo = np.maximum(t(0), lo - pos)
    over_hi = np.maximum(t(0), pos - hi)
    inv_mass = t(1.0) / st.mass
    denom = inv_mass[:, None] + np.zeros_like(pos)
    denom = np.where(denom == 0, t(1), denom)
    delta = np.maximum(over_lo, over_hi)
    wall_sign = (over_lo > 0).astype(pos.dtype) - (over_hi > 0).astype(pos.dtype)
    active = np.abs(wall_sign)
    v_contact_step = st.vel
    acc = st.force * inv_mass[:, None]
    alpha = verlet_collision_fraction(v_contact_step, acc, delta, wall_sign, sy.dt)
    alpha_min = np.min(np.where(active > 0, alpha, t(1)), axis=-1, keepdims=True)
    dt_factor = (alpha_min - t(1)) * sy.dt
    v_contact = v_contact_step + dt_factor * acc
    j_mag = -(t(1) + e) * v_contact / denom
    closing = (v_contact * wall_sign) < 0
    count_safe = np.maximum(active, t(1))
    weight = active / count_safe
    j_mag = j_mag * (weight * closing.astype(pos.dtype))
    dv = j_mag * inv_mass[:, None]
    dv = np.where(st.fixed[:, None], t(0), dv)
    st.vel = st.vel + dv
    dt_rem = (t(1) - alpha_min) * sy.dt
    # q <- unit(dq @ q) with dq = from_small_rotvec(0) = (1, 0): reflect.py:291-294
    st.q = quat_unit(quat_mul(np.concatenate([np.ones_like(st.q[:, :1]), np.zeros_like(st.q[:, 1:])], 1), st.q))
    st.pos_c = st.pos_c + dv * dt_rem
    return st


def _segment(values, ids, n, op):
    """``jax.ops.segment_{sum,max,min}`` over the leading axis, in index order."""
    if op == "sum":
        out = np.zeros((n,) + values.shape[1:], values.dtype)
        for i in range(values.shape[0]):
            out[ids[i]] = out[ids[i]] + values[i]
        return out
    init = -np.inf if op == "max" else np.inf
    out = np.full((n,) + values.shape[1:], init, values.dtype)
    f = np.maximum if op == "max" else np.minimum
    for i in range(values.shape[0]):
        out[ids[i]] = f(out[ids[i]], values[i])
    return out


def reflect_apply_clumps(st: OState, sy: OSystem):
    """``ReflectDomain.apply`` (``domains/reflect.py:99-299``) for rigid clumps: the
    clump's deepest overshoot per axis, the Verlet collision fraction of each active
    member's contact point and the clump minimum, impulses shared by the active members,
    linear and angular velocity changes summed over the clump, then the position and
    orientation corrections over the rest of the step."""
    t = st.pos_c.dtype.type
    N, d = st.N, st.dim
    cid = st.clump_id
    e = t(sy.restitution)
    dt = sy.dt
    pos_p_lab = pos_p_rot(st)
    pos = st.pos_c + pos_p_lab
    rad = st.rad[:, None]
    lo = sy.anchor + rad
    hi = sy.anchor + sy.box_size - rad
    over_lo = np.maximum(t(0), lo - pos)
    over_hi = np.maximum(t(0), pos - hi)
    max_lo = _segment(over_lo, cid, N, "max")[cid]
    max_hi = _segment(over_hi, cid, N, "max")[cid]
    inv_mass = t(1.0) / st.mass
    inv_inertia = t(1.0) / st.inertia
    eye = np.eye(d, dtype=st.pos_c.dtype)
    # n_prime[:, a, :] = rotate_back(q, e_a): the rows of the rotation matrix
    n_prime = np.stack([quat_rotate_back(st.q, np.broadcast_to(eye[a], (N, d)).copy()) for a in range(d)], 1)
    if d == 3:
        rpcn = np.stack([cross3(st.pos_p, n_prime[:, a, :]) for a in range(3)], 1)
    else:
        rpcn = np.stack([st.pos_p[:, 0:1] * n_prime[:, a, 1:2] - st.pos_p[:, 1:2] * n_prime[:, a, 0:1]
                         for a in range(2)], 1)
    denom_rot = np.einsum("ni,nji->nj", inv_inertia, rpcn * rpcn).astype(st.pos_c.dtype)
    denom = inv_mass[:, None] + denom_rot
    denom = np.where(denom == 0, t(1), denom)
    delta = np.maximum(max_lo, max_hi)
    deep_lo = (over_lo > 0) & (over_lo == max_lo)
    deep_hi = (over_hi > 0) & (over_hi == max_hi)
    wall_sign = deep_lo.astype(st.pos_c.dtype) - deep_hi.astype(st.pos_c.dtype)
    active = np.abs(wall_sign)
    v_contact_step = st.vel + _cross_w(st.ang_vel, pos_p_lab)
    acc_clump = st.force * inv_mass[:, None]
    if d == 3:
        Rm = n_prime
        RT = np.swapaxes(n_prime, -1, -2)
        tb = np.einsum("nij,nj->ni", RT, st.torque).astype(st.pos_c.dtype)
        wb = np.einsum("nij,nj->ni", RT, st.ang_vel).astype(st.pos_c.dtype)
        ab = (tb - cross3(wb, st.inertia * wb)) * inv_inertia
        alpha_rot = np.einsum("nij,nj->ni", Rm, ab).astype(st.pos_c.dtype)
    else:
        alpha_rot = st.torque * inv_inertia
    acc_contact = acc_clump + _cross_w(alpha_rot, pos_p_lab)
    alpha = verlet_collision_fraction(v_contact_step, acc_contact, delta, wall_sign, dt)
    alpha_min_dim = np.min(np.where(active > 0, alpha, t(1)), axis=-1, keepdims=True)
    alpha_clump = _segment(alpha_min_dim, cid, N, "min")[cid]
    dt_factor = (alpha_clump - t(1)) * dt
    v_contact = v_contact_step + dt_factor * acc_contact
    j = -(t(1) + e) * v_contact / denom
    closing = (v_contact * wall_sign) < 0
    count_active = _segment(active, cid, N, "sum")
    weight = active / np.maximum(count_active, t(1))[cid]
    j = j * (weight * closing.astype(st.pos_c.dtype))
    dv = _segment(j * inv_mass[:, None], cid, N, "sum")[cid]
    dv = np.where(st.fixed[:, None], t(0), dv)
    st.vel = st.vel + dv
    if d == 3:
        jb = np.einsum("nij,nj->ni", RT, j).astype(st.pos_c.dtype)
        mom = cross3(st.pos_p, jb)
        dwl = np.einsum("nij,nj->ni", Rm, mom * inv_inertia).astype(st.pos_c.dtype)
    else:
        jb = np.einsum("nji,nj->ni", n_prime, j).astype(st.pos_c.dtype)
        mom = st.pos_p[:, 0:1] * jb[:, 1:2] - st.pos_p[:, 1:2] * jb[:, 0:1]
        dwl = mom * inv_inertia
    dw = _segment(dwl, cid, N, "sum")[cid]
    dw = np.where(st.fixed[:, None], t(0), dw)
    st.ang_vel = st.ang_vel + dw
    dt_rem = (t(1) - alpha_clump) * dt
    theta = dw * dt_rem
    if d == 2:
        theta = np.concatenate([np.zeros_like(theta), np.zeros_like(theta), theta], axis=-1)
    st.q = quat_unit(quat_mul(quat_from_small_rotvec(theta), st.q))
    st.pos_c = st.pos_c + dv * dt_rem
    return st


def free_apply(st: OState, sy: OSystem):
    """``FreeDomain.apply`` (``domains/free.py:40-63``): the box of pos_c -+ (norm(pos_p) + rad)."""
    t = st.pos_c.dtype.type
    if st.rigid:
        n2 = sumsq(st.pos_p)
        nrm = np.where(n2 == 0, t(0), np.sqrt(np.maximum(n2, t(1e-16))))
        rad = (nrm + st.rad)[:, None]
    else:
        rad = st.rad[:, None]
    p_min = np.min(st.pos_c - rad, axis=0)
    p_max = np.max(st.pos_c + rad, axis=0)
    sy.box_size = (p_max - p_min).astype(st.pos_c.dtype)
    sy.anchor = p_min.astype(st.pos_c.dtype)
    return st


def force_manager_apply(st: OState, sy: OSystem):
    """``ForceManager.apply`` (``forces/force_manager.py:338-425``): contact + gravity *
    (mass / count) per sphere, then the clump sums (``segment_sum`` over clump_id, members
    added in index order) broadcast back to every member."""
    t = st.pos_c.dtype.type
    count = np.bincount(st.clump_id, minlength=st.N)[st.clump_id].astype(st.pos_c.dtype)
    F_com = sy.gravity.astype(st.pos_c.dtype) * (st.mass / count)[:, None]
    F_part = np.zeros_like(st.force)
    F_total = st.force + F_part + F_com
    T_total = st.torque + np.zeros_like(st.torque)
    if not st.rigid:
        st.force, st.torque = F_total, T_total
        return st
    F_c = np.zeros_like(F_total)
    T_c = np.zeros_like(T_total)
    for i in range(st.N):  # index order: the engine's member order
        F_c[st.clump_id[i]] = F_c[st.clump_id[i]] + F_total[i]
        T_c[st.clump_id[i]] = T_c[st.clump_id[i]] + T_total[i]
    st.force, st.torque = F_c[st.clump_id], T_c[st.clump_id]
    return st


def _kick_scale(st: OState, sy: OSystem, factor):
    t = st.pos_c.dtype.type
    return (sy.dt * t(factor) / st.mass)[:, None]


def vv_before(st: OState, sy: OSystem):
    """``VelocityVerlet.step_before_force`` (``integrators/velocity_verlet.py:29-61``)."""
    free = (~st.fixed)[:, None].astype(st.pos_c.dtype)
    st.vel = st.vel + st.force * _kick_scale(st, sy, 0.5) * free
    st.pos_c = st.pos_c + sy.dt * st.vel
    return st


def vv_after(st: OState, sy: OSystem):
    """``VelocityVerlet.step_after_force`` (``integrators/velocity_verlet.py:66-95``)."""
    free = (~st.fixed)[:, None].astype(st.pos_c.dtype)
    st.vel = st.vel + st.force * _kick_scale(st, sy, 0.5) * free
    return st


def euler_after(st: OState, sy: OSystem):
    """``DirectEuler.step_after_force`` (``integrators/direct_euler.py:30-66``)."""
    t = st.pos_c.dtype.type
    free = (~st.fixed)[:, None].astype(st.pos_c.dtype)
    st.vel = st.vel + st.force * (sy.dt / st.mass)[:, None] * free
    st.pos_c = st.pos_c + sy.dt * st.vel
    return st


# --- quaternions (utils/quaternion.py) -------------------------------------


def cross3(a, b):
    """``cross`` (``utils/linalg.py``) for 3-vectors: a_left*b_right - a_right*b_left."""
    return np.stack([
        a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1],
        a[..., 2] * b[..., 0] - a[..., 0] * b[..., 2],
        a[..., 0] * b[..., 1] - a[..., 1] * b[..., 0],
    ], axis=-1)


def dot3(a, b):
    return a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1] + a[..., 2] * b[..., 2]


def quat_unit(q):
    """``Quaternion.unit`` (``quaternion.py:75-95``)."""
    t = q.dtype.type
    n2 = q[:, 0] * q[:, 0] + dot3(q[:, 1:], q[:, 1:])
    safe = np.where(n2 == 0, t(1), n2)
    inv = t(1) / np.sqrt(safe)
    return q * inv[:, None]


def quat_mul(a, b):
    """Hamilton product ``Quaternion.__matmul__`` (``quaternion.py:347-367``)."""
    w = a[:, :1] * b[:, :1] - dot3(a[:, 1:], b[:, 1:])[:, None]
    xyz = a[:, :1] * b[:, 1:] + b[:, :1] * a[:, 1:] + cross3(a[:, 1:], b[:, 1:])
    return np.concatenate([w, xyz], axis=1)


def quat_from_small_rotvec(rv):
    """``Quaternion.from_small_rotvec`` (``quaternion.py:132-143``)."""
    t = rv.dtype.type
    n2 = dot3(rv, rv)
    c = t(1.0) - n2 / t(8.0)
    s = t(0.5) - n2 / t(48.0)
    return np.concatenate([c[:, None], rv * s[:, None]], axis=1)


def quat_rotate(q, v):
    """``Quaternion.rotate`` (``quaternion.py:193-244``)."""
    t = q.dtype.type
    if v.shape[-1] == 2:
        qw, qz = q[:, :1], q[:, 3:4]
        c = qw * qw - qz * qz
        s = t(2.0) * qw * qz
        return np.concatenate([c * v[:, :1] - s * v[:, 1:2], s * v[:, :1] + c * v[:, 1:2]], 1)
    tt = t(2.0) * cross3(q[:, 1:], v)
    return v + q[:, :1] * tt + cross3(q[:, 1:], tt)


def quat_rotate_back(q, v):
    """``Quaternion.rotate_back`` (``quaternion.py:247-270``): rotate by the conjugate."""
    qc = q.copy()
    qc[:, 1:] = -qc[:, 1:]
    return quat_rotate(qc, v)


def omega_dot(w, torque, inertia, inv_inertia):
    """``omega_dot`` (``integrators/spiral.py:22-40``)."""
    if w.shape[-1] == 3:
        wx, wy, wz = w[:, 0:1], w[:, 1:2], w[:, 2:3]
        ix, iy, iz = inertia[:, 0:1], inertia[:, 1:2], inertia[:, 2:3]
        tx, ty, tz = torque[:, 0:1], torque[:, 1:2], torque[:, 2:3]
        cx = wy * (iz * wz) - wz * (iy * wy)
        cy = wz * (ix * wx) - wx * (iz * wz)
        cz = wx * (iy * wy) - wy * (ix * wx)
        return np.concatenate([tx - cx, ty - cy, tz - cz], axis=1) * inv_inertia
    return torque * inv_inertia


def _ssprk3(st: OState, sy: OSystem, h):
    t = st.pos_c.dtype.type
    inv_i = t(1.0) / st.inertia
    if st.dim == 3:
        w = quat_rotate_back(st.q, st.ang_vel)
        tq = quat_rotate_back(st.q, st.torque)
    else:
        w, tq = st.ang_vel, st.torque
    k1 = h * omega_dot(w, tq, st.inertia, inv_i)
    k2 = h * omega_dot(w + k1, tq, st.inertia, inv_i)
    k3 = h * omega_dot(w + t(0.25) * (k1 + k2), tq, st.inertia, inv_i)
    free = (~st.fixed)[:, None].astype(st.pos_c.dtype)
    w = w + free * (k1 + k2 + t(4.0) * k3) / t(6.0)
    return w


def vvspiral_before(st: OState, sy: OSystem):
    """``VelocityVerletSpiral.step_before_force`` (``velocity_verlet_spiral.py:36-116``)."""
    t = st.pos_c.dtype.type
    dt_2 = sy.dt / t(2.0)
    w = _ssprk3(st, sy, dt_2)
    rotvec = t(2.0) * dt_2 * w
    if st.dim == 2:
        rotvec = np.array([0.0, 0.0, 1.0], st.pos_c.dtype) * rotvec
    dq = quat_from_small_rotvec(rotvec)
    st.q = quat_unit(quat_mul(st.q, dq))
    st.ang_vel = quat_rotate(st.q, w) if st.dim == 3 else w
    return st


def vvspiral_after(st: OState, sy: OSystem):
    """``VelocityVerletSpiral.step_after_force`` (``velocity_verlet_spiral.py:121-180``)."""
    t = st.pos_c.dtype.type
    dt_2 = sy.dt / t(2.0)
    w = _ssprk3(st, sy, dt_2)
    st.ang_vel = quat_rotate(st.q, w) if st.dim == 3 else w
    return st


def spiral_after(st: OState, sy: OSystem):
    """``Spiral.step_after_force`` (``integrators/spiral.py:56-144``)."""
    t = st.pos_c.dtype.type
    dt_2 = sy.dt / t(2)
    inv_i = t(1.0) / st.inertia
    if st.dim == 3:
        w = quat_rotate_back(st.q, st.ang_vel)
        tq = quat_rotate_back(st.q, st.torque)
    else:
        w, tq = st.ang_vel, st.torque
    w_dot = omega_dot(w, tq, st.inertia, inv_i)
    rv1 = t(2.0) * dt_2 * w
    rv2 = t(2.0) * dt_2 * dt_2 * w_dot
    if st.dim == 2:
        ez = np.array([0.0, 0.0, 1.0], st.pos_c.dtype)
        rv1, rv2 = ez * rv1, ez * rv2
    dq = quat_mul(quat_from_small_rotvec(rv1), quat_from_small_rotvec(rv2))
    st.q = quat_unit(quat_mul(st.q, dq))
    k1 = sy.dt * w_dot
    k2 = sy.dt * omega_dot(w + k1, tq, st.inertia, inv_i)
    k3 = sy.dt * omega_dot(w + t(0.25) * (k1 + k2), tq, st.inertia, inv_i)
    free = (~st.fixed)[:, None].astype(st.pos_c.dtype)
    w = w + free * (k1 + k2 + t(4.0) * k3) / t(6.0)
    st.ang_vel = quat_rotate(st.q, w) if st.dim == 3 else w
    return st


# ---------------------------------------------------------------------------
# Step driver.
# ---------------------------------------------------------------------------


def step_once(st: OState, sy: OSystem, sum_dtype=None, collider="celllist"):
    """``_step_once`` (``system.py:60-82``) with the fixed stage order."""
    t = st.pos_c.dtype.type
    sy.time = t(sy.time + sy.dt)
    sy.step_count += 1
    if sy.domain == "reflect":
        st = reflect_apply(st, sy)
    elif sy.domain == "free":
        st = free_apply(st, sy)
    sy.inv_box_size = (t(1.0) / sy.box_size).astype(st.pos_c.dtype)
    if sy.linear == "verlet":
        st = vv_before(st, sy)
    if sy.rotation == "verletspiral":
        st = vvspiral_before(st, sy)
    if collider == "naive" and sy.force_law != "cundallstrack":
        st.force = naive_force(st, sy)
        st.torque = np.zeros_like(st.torque)
    else:
        st.force, st.torque = collider_force(st, sy, sum_dtype)
    st = force_manager_apply(st, sy)
    if sy.linear == "verlet":
        st = vv_after(st, sy)
    elif sy.linear == "euler":
        st = euler_after(st, sy)
    if sy.rotation == "verletspiral":
        st = vvspiral_after(st, sy)
    elif sy.rotation == "spiral":
        st = spiral_after(st, sy)
    return st, sy


def step(st: OState, sy: OSystem, n: int, **kw):
    """``System.step`` (``system.py:701-748``): ``n`` applications of ``_step_once``."""
    for _ in range(int(n)):
        st, sy = step_once(st, sy, **kw)
    return st, sy


# ---------------------------------------------------------------------------
# Energy, contacts, neighbour list.
# ---------------------------------------------------------------------------


def naive_energy(st: OState, sy: OSystem) -> float:
    """Collider PE over all pairs (``colliders/naive.py``; pair term x0.5, ``_partition.py:39-51``)."""
    N = st.N
    ii, jj = np.meshgrid(np.arange(N), np.arange(N), indexing="ij")
    ii, jj = ii.ravel(), jj.ravel()
    e = pair_energy(ii, jj, world_pos(st), st.rad, st.mat_id, sy)
    ok = valid_mask(st.clump_id[ii], st.clump_id[jj], st.bond_id[ii], jj, sy.interact_same_bond_id)
    return float(np.sum(np.where(ok, st.pos_c.dtype.type(0.5) * e, 0).astype(np.float64)))


def compute_energy(st: OState, sy: OSystem, naive: bool = False):
    """``thermal.compute_energy`` (``utils/thermal.py:153-177``), accumulated in float64.

    Returns ``(pe_pair, pe_gravity, ke_trans, ke_rot)``.
    """
    pe_pair = naive_energy(st, sy) if naive else cell_list_energy(st, sy, sum_dtype=np.float64)
    # clump members carry the clump's mass and inertia: each counts 1 / count
    # (thermal.py:24-80, force_manager.py:427-459)
    count = np.bincount(st.clump_id, minlength=st.N)[st.clump_id].astype(np.float64)
    w = st.mass.astype(np.float64) / count
    g = sy.gravity.astype(np.float64)
    pe_grav = -float(np.sum((st.pos_c.astype(np.float64) @ g) * w))
    ke_t = float(np.sum(0.5 * w * np.sum(st.vel.astype(np.float64) ** 2, axis=1)))
    if st.dim == 3:
        wb = quat_rotate_back(st.q, st.ang_vel).astype(np.float64)
    else:
        wb = st.ang_vel.astype(np.float64)
    ke_r = float(np.sum(0.5 * np.sum(wb * (st.inertia.astype(np.float64) * wb), axis=1) / count))
    return pe_pair, pe_grav, ke_t, ke_r


def contact_pairs(st: OState, sy: OSystem):
    """Canonical contact set: sorted ``(i < j)`` pairs with ``d_sq < (ri + rj)^2``.

    The reference has no contact-set API; ``utils/contacts.py:21-86`` keeps
    the candidate slots whose spring force is nonzero, i.e. overlap > 0.  The
    canonical predicate compares the squared distance (``forces/spring.py:
    97-99`` arithmetic, left-to-right sum, no FMA) with the squared contact
    distance so that oracle and kernel evaluate identical IEEE operations.
    All pairs are enumerated through the cell list, so only pairs inside one
    stencil are considered, as in the reference.
    """
    N = st.N
    pos = world_pos(st)
    cell = np.float32(2.0) * st.rad.max()
    sy2 = replace(sy)
    sy2.inv_box_size = sy.inv_box_size
    g, strides, cellv, _ = grid_params(sy.box_size, cell, sy.periodic)
    # brute force in blocks: exact for any N the tests use
    out = []
    B = 2048
    for a in range(0, N, B):
        ii = np.arange(a, min(N, a + B))
        rij = displacement_fast(pos[ii][:, None, :], pos[None, :, :], sy)
        d_sq = sumsq(rij)
        R = st.rad[ii][:, None] + st.rad[None, :]
        hit = d_sq < R * R
        jj = np.arange(N)[None, :]
        hit &= jj > ii[:, None]
        hit &= st.clump_id[ii][:, None] != st.clump_id[None, :]  # one clump: no contact
        bi, bj = np.nonzero(hit)
        out.append(np.stack([ii[bi], bj], 1))
    pairs = np.concatenate(out, 0) if out else np.zeros((0, 2), np.int64)
    order = np.lexsort((pairs[:, 1], pairs[:, 0]))
    return pairs[order].astype(np.int64)


def create_neighbor_list(st: OState, sy: OSystem, cutoff, max_neighbors):
    """``DynamicCellList.create_neighbor_list`` (``colliders/cell_list.py:498-595``).

    Cell size inflated to cover the cutoff (``:537-538``), per-stencil-cell
    scan (``_make_stencil_body`` ``:99-174``) with ``d_sq <= cutoff^2`` on the
    true-division displacement (``periodic.py:37-71``), prefix-sum packing
    (``_partition.py:102-150``), indices mapped back through ``perm``.
    Positions are ``state.pos`` (members' world positions for clumps; members of one
    clump never list each other).  Returns ``(nl (N, max_neighbors) int, overflow bool)``.
    """
    N = st.N
    pos = world_pos(st)
    t = pos.dtype.type
    cutoff_sq = t(cutoff) * t(cutoff)
    if max_neighbors == 0:
        return np.zeros((N, 0), np.int64), False
    sr = max(int(np.max(sy.neighbor_mask)), 1)
    cell_size = np.maximum(sy.cell_size, t(cutoff) / t(sr)).astype(pos.dtype)
    perm, sorted_h, nh = spatial_partition(pos, sy, cell_size, sy.neighbor_mask)
    if sy.periodic:
        nh = dedup_stencil_exact(nh)
    nl = np.full((N, max_neighbors), -1, np.int64)
    overflow = False
    for i in range(N):
        cnt = 0
        for m in range(nh.shape[1]):
            h = nh[i, m]
            if h == -1:
                continue
            k = int(np.searchsorted(sorted_h, h, side="left"))
            c_local = 0
            while k < N and sorted_h[k] == h:
                j = perm[k]
                dr = displacement_true(pos[i], pos[j], sy)
                ok = valid_mask(st.clump_id[j], st.clump_id[i], st.bond_id[j][None, :],
                                np.array([i]), sy.interact_same_bond_id)[0]
                if ok and sumsq(dr[None, :])[0] <= cutoff_sq:
                    if c_local < max_neighbors:
                        if cnt < max_neighbors:
                            nl[i, cnt] = j
                    else:
                        overflow = True
                    c_local += 1
                    cnt += 1
                k += 1
        if cnt > max_neighbors:
            overflow = True
    return nl, overflow
