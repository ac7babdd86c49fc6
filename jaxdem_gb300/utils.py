"""Energy and contact utilities (``jaxdem/utils/thermal.py``, ``jaxdem/utils/contacts.py``).

Energies and neighbour lists are evaluated by the GB300 engine; the per-pair
force of ``get_pair_forces_and_ids`` is restated on the host from the device
neighbour list with the same float32 operations as ``spring.py:97-108`` or
``hertz.py:99-117``.
"""

from __future__ import annotations

import numpy as np

from . import session

F32 = np.float32


def compute_potential_energy(state, system):
    """Collider + force-manager potential energy (``thermal.py:125-150``)."""
    e = session.energies(state, system)
    return (e[..., 0] + e[..., 1]).astype(F32) if np.ndim(e) > 1 else F32(e[0] + e[1])


def compute_translational_kinetic_energy(state):
    v = np.asarray(state.vel, np.float64)
    return F32(np.sum(0.5 * np.asarray(state.mass, np.float64) * np.sum(v * v, axis=-1)))


def compute_energy(state, system):
    """``compute_energy`` (``thermal.py:153-177``): PE + translational + rotational KE."""
    e = session.energies(state, system)
    tot = e[..., 0] + e[..., 1] + e[..., 2] + e[..., 3]
    return tot.astype(F32) if np.ndim(tot) else F32(tot)


def energy_terms(state, system) -> np.ndarray:
    """``(pe_collider, pe_gravity, ke_trans, ke_rot)`` in float64."""
    return session.energies(state, system)


def contact_pairs(state, system) -> np.ndarray:
    """Sorted ``(i < j)`` pairs with positive spring overlap (device cell list)."""
    return session.contacts(state, system)


def get_pair_forces_and_ids(state, system, cutoff=None, max_neighbors=None):
    """``get_pair_forces_and_ids`` (``contacts.py:21-86``)."""
    if cutoff is None:
        cutoff = float(np.max(state.rad)) * 3.0
    if max_neighbors is None:
        max_neighbors = 100
    state, system, nl, overflow = system.collider.create_neighbor_list(state, system, cutoff, max_neighbors)
    if overflow:
        raise ValueError("Neighbor list overflowed. Increase max_neighbors.")
    N, d = state.N, state.dim
    pos = state.pos
    i_ids = np.repeat(np.arange(N)[:, None], nl.shape[1], axis=1).ravel()
    j_ids = nl.ravel()
    valid = j_ids != -1
    sj = np.maximum(j_ids, 0)
    rij = pos[i_ids] - pos[sj]
    if system.domain.periodic:
        rij = (rij - system.domain.box_size * np.round(rij * system.domain.inv_box_size)).astype(F32)
    d_sq = rij[:, 0] * rij[:, 0]
    for a in range(1, d):
        d_sq = d_sq + rij[:, a] * rij[:, a]
    ri, rj = state.rad[i_ids], state.rad[sj]
    R = ri + rj
    law, table, props = session.pair_law(system)
    if law == "cundallstrack":
        f = _cundall_strack_pairs(state, i_ids, sj, rij, table, props) * valid[:, None]
        return state, system, np.column_stack((i_ids, j_ids)), f.astype(F32)
    k = table[state.mat_id[i_ids], state.mat_id[sj]]
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = np.where(d_sq == 0, F32(0), F32(1) / np.sqrt(np.maximum(d_sq, F32(1e-16))))
    r = d_sq * inv
    delta = np.maximum(F32(0), R - r) * (i_ids != sj).astype(F32)
    if law == "hertz":
        # hertz.py:99-117: k = (4/3) E* sqrt(R*), F = k delta^(3/2) (r_ij / r)
        with np.errstate(divide="ignore", invalid="ignore"):
            kk = k * np.sqrt((ri * rj) / R)
        mag = np.where(valid, kk * np.power(delta, F32(1.5)), F32(0))
        f = (mag[:, None] * (rij * inv[:, None])).astype(F32) * valid[:, None]
    else:
        f = ((k * delta * inv)[:, None] * rij).astype(F32) * valid[:, None]
    return state, system, np.column_stack((i_ids, j_ids)), f.astype(F32)


def _cundall_strack_pairs(state, i, j, rij, beta, props):
    """Contact force on i due to j of ``CundallStrackForce.force``
    (``cundall_strack.py:100-196``) for the listed pairs, float32."""
    d = rij.shape[1]
    mi, mj = state.mat_id[i], state.mat_id[j]
    Ei, Ej, Gi, Gj = props[mi, 0], props[mj, 0], props[mi, 1], props[mj, 1]
    Ri, Rj = state.rad[i], state.rad[j]
    m_i, m_j = state.mass[i], state.mass[j]
    kn = (F32(2.0) * Ei * Ri * Ej * Rj) / (Ei * Ri + Ej * Rj)
    kt = (F32(2.0) * Gi * Ri * Gj * Rj) / (Gi * Ri + Gj * Rj)
    m_eff = (m_i * m_j) / (m_i + m_j)
    mu_eff = np.minimum(props[mi, 2], props[mj, 2])
    b = beta[mi, mj]
    gamma_n = F32(2.0) * b * np.sqrt(kn * m_eff)
    gamma_t = F32(2.0) * b * np.sqrt(kt * m_eff)

    def unit_and_norm(v):
        n2 = np.sum(v * v, axis=1, dtype=F32)
        with np.errstate(divide="ignore"):
            inv = np.where(n2 == 0, F32(0), F32(1) / np.sqrt(np.maximum(n2, F32(1e-16))))
        return v * inv[:, None], n2 * inv

    n, r = unit_and_norm(rij)
    delta = Ri + Rj - r
    contact = ((delta > 0) & (i != j)).astype(F32)
    delta = delta * contact
    w = np.asarray(state.ang_vel, F32)

    def w_cross(wv, rv):
        if d == 3:
            return np.cross(wv, rv).astype(F32)
        return np.stack([-wv[:, 0] * rv[:, 1], wv[:, 0] * rv[:, 0]], 1)

    v_ci = state.vel[i] + w_cross(w[i], -Ri[:, None] * n)
    v_cj = state.vel[j] + w_cross(w[j], Rj[:, None] * n)
    v_rel = v_ci - v_cj
    vn = np.sum(v_rel * n, axis=1, dtype=F32)
    t, vt = unit_and_norm(v_rel - vn[:, None] * n)
    Fn = np.maximum(F32(0), kn * delta - gamma_n * vn) * contact
    Ft = np.minimum(gamma_t * vt, mu_eff * Fn) * contact
    return (Fn[:, None] * n - Ft[:, None] * t).astype(F32)


def grid_state(*, n_per_axis, spacing, radius: float = 1.0, mass: float = 1.0, jitter: float = 0.0,
               vel_range=None, radius_range=None, mass_range=None, seed: int = 0):
    """Particles on a rectangular lattice (``utils/grid_state.py:21-130``).

    Same lattice (``meshgrid(indexing="ij")`` of ``arange(n) * spacing``) and
    the same uniform ranges; random draws come from numpy's PCG64 instead of
    JAX's PRNG, so the values differ from the reference's for equal seeds.
    """
    from .state import State

    n_per_axis = tuple(int(n) for n in n_per_axis)
    dim = len(n_per_axis)
    sp = (float(spacing),) * dim if np.isscalar(spacing) else tuple(float(s) for s in spacing)
    axes = [np.arange(n) * s for n, s in zip(n_per_axis, sp)]
    coords = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1).reshape(-1, dim).astype(F32)
    rng = np.random.Generator(np.random.PCG64(seed))
    N = coords.shape[0]
    if jitter > 0:
        coords = (coords + rng.uniform(-jitter, jitter, coords.shape)).astype(F32)
    rad = (rng.uniform(radius_range[0], radius_range[1], N) if radius_range is not None
           else np.full(N, radius)).astype(F32)
    m = (rng.uniform(mass_range[0], mass_range[1], N) if mass_range is not None else np.full(N, mass)).astype(F32)
    vr = (-1.0, 1.0) if vel_range is None else tuple(vel_range)
    vel = rng.uniform(vr[0], vr[1], coords.shape).astype(F32)
    return State.create(pos=coords, vel=vel, rad=rad, mass=m)
