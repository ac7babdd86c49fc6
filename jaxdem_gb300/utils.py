"""Energy and contact utilities (``jaxdem/utils/thermal.py``, ``jaxdem/utils/contacts.py``).

Energies and neighbour lists are evaluated by the GB300 engine; the per-pair
spring force of ``get_pair_forces_and_ids`` is restated on the host from the
device neighbour list with the same float32 operations as ``spring.py:97-108``.
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
    R = state.rad[i_ids] + state.rad[sj]
    k = np.asarray(system.mat_table.young_eff, F32)[state.mat_id[i_ids], state.mat_id[sj]]
    with np.errstate(divide="ignore"):
        inv = np.where(d_sq == 0, F32(0), F32(1) / np.sqrt(np.maximum(d_sq, F32(1e-16))))
    r = d_sq * inv
    delta = np.maximum(F32(0), R - r) * (i_ids != sj).astype(F32)
    f = ((k * delta * inv)[:, None] * rij).astype(F32) * valid[:, None]
    return state, system, np.column_stack((i_ids, j_ids)), f.astype(F32)
