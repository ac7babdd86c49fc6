"""Particle state, mirroring ``jaxdem.State`` (``jaxdem/state.py``) for spheres.

Fields, shapes and ``State.create`` defaults follow ``state.py:103-228`` and
``state.py:369-867``; arrays are numpy float32 / int32 on the host.  The
device copy lives in the engine handle (``include/jdem_gb300.h``) between
calls.  A leading batch axis ``(B, N, ...)`` marks independent systems,
as ``jax.vmap`` batching does in the reference (``system.py:743-744``).
"""

from __future__ import annotations

from dataclasses import dataclass, field, fields, replace
from typing import Any, Optional, Sequence

import numpy as np

F32 = np.float32


@dataclass
class Quaternion:
    """Orientation ``(w, xyz)`` with ``w`` (..., 1) and ``xyz`` (..., 3) (``utils/quaternion.py``)."""

    w: np.ndarray
    xyz: np.ndarray

    @staticmethod
    def create(w=None, xyz=None) -> "Quaternion":
        w = np.ones((1, 1), F32) if w is None else np.asarray(w, F32)
        xyz = np.zeros((1, 3), F32) if xyz is None else np.asarray(xyz, F32)
        return Quaternion(w, xyz)

    def as_array(self) -> np.ndarray:
        """(..., 4) array ``[w, x, y, z]``."""
        return np.concatenate([self.w, self.xyz], axis=-1).astype(F32)

    @staticmethod
    def from_array(q: np.ndarray) -> "Quaternion":
        q = np.asarray(q, F32)
        return Quaternion(q[..., 0:1].copy(), q[..., 1:].copy())


def _hypersphere_volume(rad: np.ndarray, dim: int) -> np.ndarray:
    if dim == 2:
        return (F32(np.pi) * rad * rad).astype(F32)
    return (F32(4.0 / 3.0) * F32(np.pi) * rad * rad * rad).astype(F32)


def _symmetrize_bonds(conn: np.ndarray, N: int) -> np.ndarray:
    """Symmetric, -1 padded (N, W) bond table (``state.py:735-761``)."""
    w = max(conn.shape[-1], 1)
    rows = np.repeat(np.arange(N), conn.shape[-1])
    cols = conn.reshape(-1)
    ok = (cols >= 0) & (cols < N)
    i, j = rows[ok], cols[ok]
    if i.size == 0:
        return np.full((N, w), -1, np.int32)
    pairs = np.unique(np.stack((np.concatenate((i, j)), np.concatenate((j, i))), 1), axis=0)
    counts = np.bincount(pairs[:, 0], minlength=N)
    deg = max(int(counts.max()), w)
    out = np.full((N, deg), -1, np.int32)
    starts = np.cumsum(counts) - counts
    slot = np.arange(pairs.shape[0]) - starts[pairs[:, 0]]
    out[pairs[:, 0], slot] = pairs[:, 1]
    return out


@dataclass
class State:
    pos_c: np.ndarray
    pos_p: np.ndarray
    vel: np.ndarray
    force: np.ndarray
    q: Quaternion
    ang_vel: np.ndarray
    torque: np.ndarray
    rad: np.ndarray
    _rad: np.ndarray
    volume: np.ndarray
    mass: np.ndarray
    inertia: np.ndarray
    clump_id: np.ndarray
    bond_id: np.ndarray
    mat_id: np.ndarray
    species_id: np.ndarray
    fixed: np.ndarray
    facet_id: np.ndarray = field(default_factory=lambda: np.zeros((0,), np.int32))

    # -- shape helpers (state.py:275-304) ---------------------------------
    @property
    def N(self) -> int:
        return self.pos_c.shape[-2]

    @property
    def dim(self) -> int:
        return self.pos_c.shape[-1]

    @property
    def shape(self) -> tuple:
        return self.pos_c.shape

    @property
    def batch_size(self) -> int:
        return 1 if self.pos_c.ndim < 3 else self.pos_c.shape[-3]

    @property
    def _pos_p_rot(self) -> np.ndarray:
        return _rotate(self.q, self.pos_p)

    @property
    def pos(self) -> np.ndarray:
        """``pos_c + R(q) pos_p`` (``state.py:295-304``)."""
        return (self.pos_c + self._pos_p_rot).astype(F32)

    def copy(self) -> "State":
        kw = {}
        for f in fields(self):
            v = getattr(self, f.name)
            kw[f.name] = Quaternion(v.w.copy(), v.xyz.copy()) if isinstance(v, Quaternion) else np.array(v, copy=True)
        return State(**kw)

    # -- construction ------------------------------------------------------
    @staticmethod
    def create(pos=None, *, dim: Optional[int] = None, pos_p=None, vel=None, force=None, q=None, ang_vel=None,
               torque=None, rad=None, _rad=None, volume=None, mass=None, inertia=None, clump_id=None,
               bond_id=None, mat_id=None, species_id=None, fixed=None, facet_id=None, facet_vertices=None,
               mat_table=None) -> "State":
        """Defaults of ``State.create`` (``state.py:640-862``)."""
        if pos is None:
            d = 3 if dim is None else int(dim)
            pos = np.zeros((0, d), F32)
        pos_c = np.asarray(pos, F32)
        if pos_c.ndim < 2 or pos_c.shape[-1] not in (2, 3):
            raise ValueError(f"`pos` must have shape (..., N, 2|3), got {pos_c.shape}")
        lead = pos_c.shape[:-1]
        N, d = pos_c.shape[-2], pos_c.shape[-1]
        ad = 1 if d == 2 else 3
        ang_shape = (*lead, ad)
        pos_p = np.zeros_like(pos_c) if pos_p is None else np.asarray(pos_p, F32)
        vel = np.zeros_like(pos_c) if vel is None else np.asarray(vel, F32)
        force = np.zeros_like(pos_c) if force is None else np.asarray(force, F32)
        if q is None:
            qq = Quaternion(np.ones((*lead, 1), F32), np.zeros((*lead, 3), F32))
        elif isinstance(q, Quaternion):
            qq = q
        else:
            qq = Quaternion.from_array(np.asarray(q, F32))
        ang_vel = np.zeros(ang_shape, F32) if ang_vel is None else np.asarray(ang_vel, F32)
        torque = np.zeros_like(ang_vel) if torque is None else np.asarray(torque, F32)
        rad = np.ones(lead, F32) if rad is None else np.asarray(rad, F32)
        volume = _hypersphere_volume(rad, d) if volume is None else np.asarray(volume, F32)
        clump_id = np.broadcast_to(np.arange(N, dtype=np.int32), lead).copy() if clump_id is None \
            else np.asarray(clump_id, np.int32)
        if bond_id is None:
            bond = np.full((*lead, 1), -1, np.int32)
        else:
            try:
                conn = np.asarray(bond_id, np.int64)
                if conn.ndim == len(lead):
                    conn = conn[..., None]
            except (ValueError, TypeError):
                rows = [[int(v) for v in (np.asarray(r).ravel().tolist() if hasattr(r, "__iter__") else [r])]
                        for r in list(bond_id)[:N]]
                width = max(max((len(r) for r in rows), default=0), 1)
                conn = np.full((N, width), -1, np.int64)
                for i, r in enumerate(rows):
                    conn[i, : len(r)] = r
            if conn.ndim == 2:
                bond = _symmetrize_bonds(conn, N)
            else:
                flat = conn.reshape((-1, *conn.shape[-2:]))
                outs = [_symmetrize_bonds(c, N) for c in flat]
                w = max(o.shape[-1] for o in outs)
                outs = [np.pad(o, ((0, 0), (0, w - o.shape[-1])), constant_values=-1) for o in outs]
                bond = np.stack(outs).reshape((*conn.shape[:-2], N, w))
        mat_id = np.zeros(lead, np.int32) if mat_id is None else np.asarray(mat_id, np.int32)
        species_id = np.zeros(lead, np.int32) if species_id is None else np.asarray(species_id, np.int32)
        fixed = np.zeros(lead, bool) if fixed is None else np.asarray(fixed, bool)
        facet_id = np.full(lead, -1, np.int32) if facet_id is None else np.asarray(facet_id, np.int32)
        if mat_table is not None:
            mass = (np.asarray(mat_table.density, F32)[mat_id] * volume).astype(F32)
        else:
            mass = np.ones(lead, F32) if mass is None else np.asarray(mass, F32)
        coeff = F32(0.5) if d == 2 else F32(0.4)
        inertia = ((coeff * mass * rad * rad)[..., None] * np.ones_like(ang_vel)).astype(F32) if inertia is None \
            else np.asarray(inertia, F32)
        if N > 0:
            flat = clump_id.reshape((-1, N))
            clump_id = np.stack([np.unique(r, return_inverse=True)[1] for r in flat]).reshape(clump_id.shape)
            clump_id = clump_id.astype(np.int32)
        _rad = rad.copy() if _rad is None else np.asarray(_rad, F32)
        return State(pos_c=pos_c.copy(), pos_p=pos_p, vel=vel.copy(), force=force.copy(), q=qq,
                     ang_vel=ang_vel.copy(), torque=torque.copy(), rad=rad.copy(), _rad=_rad, volume=volume,
                     mass=mass, inertia=inertia, clump_id=clump_id, bond_id=bond.astype(np.int32),
                     mat_id=mat_id, species_id=species_id, fixed=fixed, facet_id=facet_id)

    @staticmethod
    def merge(a: "State", b: "State") -> "State":
        """Concatenate two unbatched states along the particle axis (``state.py:868-975``):
        the second state's clump ids are shifted past the first's, its bond indices by
        the first's particle count."""
        kw = {}
        na = a.N
        for f in fields(a):
            va, vb = getattr(a, f.name), getattr(b, f.name)
            if isinstance(va, Quaternion):
                kw[f.name] = Quaternion(np.concatenate([va.w, vb.w]), np.concatenate([va.xyz, vb.xyz]))
            elif f.name == "clump_id":
                off = int(va.max()) + 1 if va.size else 0
                kw[f.name] = np.concatenate([va, vb + off]).astype(np.int32)
            elif f.name == "bond_id":
                w = max(va.shape[-1], vb.shape[-1])
                pa = np.pad(va, ((0, 0), (0, w - va.shape[-1])), constant_values=-1)
                pb = np.pad(np.where(vb >= 0, vb + na, -1), ((0, 0), (0, w - vb.shape[-1])), constant_values=-1)
                kw[f.name] = np.concatenate([pa, pb]).astype(np.int32)
            elif f.name == "facet_id" and va.shape[:1] != (na,):
                kw[f.name] = va
            else:
                kw[f.name] = np.concatenate([va, vb])
        return State(**kw)

    @staticmethod
    def add_clump(state: "State", pos, *, pos_p=None, vel=None, force=None, q=None, ang_vel=None, torque=None,
                  rad=None, volume=None, mass=None, inertia=None, bond_id=None, mat_id=None, species_id=None,
                  fixed=None) -> "State":
        """``State.add_clump`` (``state.py:1230-1420``): append one rigid clump.

        With ``pos_p`` None, ``pos`` are the spheres' absolute positions and the
        centre is their volume-weighted mean (offsets rotated back by ``q`` when
        given); otherwise ``pos`` is the centre and ``pos_p`` the body-frame
        offsets.  The clump's velocity, orientation, spin, mass, inertia and
        fixed flag are broadcast to every member (members store the clump's
        totals)."""
        pos = np.asarray(pos, F32)
        d = pos.shape[-1]
        ad = 1 if d == 2 else 3
        qobj = None
        if q is not None:
            qobj = q if isinstance(q, Quaternion) else Quaternion.from_array(np.asarray(q, F32))
        if pos_p is None:
            n_new = pos.shape[-2]
            rad_arr = np.ones(n_new, F32) if rad is None else np.asarray(rad, F32)
            vol = _hypersphere_volume(rad_arr, d)
            vsum = vol.sum(dtype=F32)
            com = (pos * vol[:, None]).sum(axis=0, dtype=F32) / (F32(1.0) if vsum == 0 else vsum)
            pos_c = np.broadcast_to(com.astype(F32), pos.shape).copy()
            raw = (pos - pos_c).astype(F32)
            if qobj is not None:
                qb = Quaternion(np.broadcast_to(qobj.w, (n_new, 1)).copy(), np.broadcast_to(qobj.xyz, (n_new, 3)).copy())
                pos_p = _rotate(Quaternion(qb.w, -qb.xyz), raw)
            else:
                pos_p = raw
        else:
            pos_p = np.asarray(pos_p, F32)
            n_new = pos_p.shape[-2]
            com = pos if pos.ndim == 1 else pos[0]
            pos_c = np.broadcast_to(np.asarray(com, F32), (n_new, d)).copy()

        def bc(v, shape, dt=F32):
            return None if v is None else np.broadcast_to(np.asarray(v, dt), shape).copy()

        if qobj is not None:
            qobj = Quaternion(np.broadcast_to(qobj.w, (n_new, 1)).copy(), np.broadcast_to(qobj.xyz, (n_new, 3)).copy())
        new = State.create(pos=pos_c, pos_p=pos_p, vel=bc(vel, (n_new, d)), force=bc(force, (n_new, d)), q=qobj,
                           ang_vel=bc(ang_vel, (n_new, ad)), torque=bc(torque, (n_new, ad)), rad=rad,
                           volume=bc(volume, (n_new,)), mass=bc(mass, (n_new,)), inertia=bc(inertia, (n_new, ad)),
                           clump_id=np.zeros(n_new, np.int32), bond_id=bond_id, mat_id=bc(mat_id, (n_new,), np.int32),
                           species_id=bc(species_id, (n_new,), np.int32), fixed=bc(fixed, (n_new,), bool))
        return State.merge(state, new)

    @staticmethod
    def stack(states: Sequence["State"]) -> "State":
        """Stack along a new leading axis (``state.py:1131-1203``)."""
        kw = {}
        for f in fields(states[0]):
            vals = [getattr(s, f.name) for s in states]
            if isinstance(vals[0], Quaternion):
                kw[f.name] = Quaternion(np.stack([v.w for v in vals]), np.stack([v.xyz for v in vals]))
            else:
                kw[f.name] = np.stack(vals)
        return State(**kw)

    def unstack(self) -> list:
        """Inverse of :meth:`stack` for a batched state."""
        out = []
        for b in range(self.batch_size):
            kw = {}
            for f in fields(self):
                v = getattr(self, f.name)
                kw[f.name] = Quaternion(v.w[b], v.xyz[b]) if isinstance(v, Quaternion) else v[b]
            out.append(State(**kw))
        return out


def _rotate(q: Quaternion, v: np.ndarray) -> np.ndarray:
    """``Quaternion.rotate`` (``quaternion.py:193-244``)."""
    if v.shape[-1] == 2:
        qw, qz = q.w, q.xyz[..., 2:3]
        c = qw * qw - qz * qz
        s = F32(2) * qw * qz
        return np.concatenate([c * v[..., 0:1] - s * v[..., 1:2], s * v[..., 0:1] + c * v[..., 1:2]], -1)
    t = F32(2) * np.cross(q.xyz, v)
    return (v + q.w * t + np.cross(q.xyz, t)).astype(F32)
