"""Bridge between the host mirror (State/System) and the device engine.

A ``System`` plus a ``State`` (optionally batched along a leading axis, one
device system per batch member) map onto one engine handle
(``include/jdem_gb300.h``).  Handles are cached by their static
configuration, so repeated ``System.step`` calls reuse device memory and
captured CUDA graphs; each call uploads the caller's state, runs, and reads
the result back (the functional contract of the reference API).

Configurations outside the GB300 hot path raise ``NotImplementedError``:
clumps (``pos_p != 0`` or shared ``clump_id``), facets, bonded force models,
force models other than ``spring``, user force functions, pending external
forces and user pre/post-step actions.
"""

from __future__ import annotations

import collections
import dataclasses
from typing import Any, Callable, Optional

import numpy as np

from ._lib import DOMAIN, LINEAR, ROTATION, Engine
from .factory import _normalize_key
from .state import Quaternion, State

F32 = np.float32

_CACHE: "collections.OrderedDict[tuple, Engine]" = collections.OrderedDict()
_CACHE_MAX = 4


def _domain_key(system) -> str:
    name = system.domain.type_name
    if name not in DOMAIN:
        raise NotImplementedError(f"domain '{name}' is not supported by the GB300 engine")
    return name


def _check_supported(state: State, system) -> None:
    if system.force_model.type_name != "spring":
        raise NotImplementedError(f"force model '{system.force_model.type_name}' is not on the GB300 hot path")
    coll = system.collider.type_name
    if coll not in ("celllist", "naive", "celllistgb300", "neighborlist"):
        raise NotImplementedError(f"collider '{coll}' is not supported by the GB300 engine")
    _domain_key(system)
    if system.linear_integrator.type_name not in LINEAR:
        raise NotImplementedError(f"linear integrator '{system.linear_integrator.type_name}'")
    if system.rotation_integrator.type_name not in ROTATION:
        raise NotImplementedError(f"rotation integrator '{system.rotation_integrator.type_name}'")
    if system.bonded_force_model is not None:
        raise NotImplementedError("bonded force models are outside the GB300 hot path")
    fm = system.force_manager
    if fm.force_functions:
        raise NotImplementedError("user force functions are outside the GB300 hot path")
    if np.any(fm.external_force) or np.any(fm.external_force_com) or np.any(fm.external_torque):
        raise NotImplementedError("pending external forces are outside the GB300 hot path")
    from .system import _save_state_system

    if system.user_pre_step_actions is not _save_state_system or system.user_post_step_actions is not _save_state_system:
        raise NotImplementedError("user pre/post step actions are outside the GB300 hot path")
    if np.any(state.pos_p != 0):
        raise NotImplementedError("clumps (pos_p != 0) are outside the GB300 hot path")
    N = state.N
    cid = state.clump_id.reshape(-1, N) if N else state.clump_id
    if N and np.any(cid != np.arange(N)):
        raise NotImplementedError("clumps (shared clump_id) are outside the GB300 hot path")
    if state.facet_id.size and np.any(state.facet_id != -1):
        raise NotImplementedError("facets are outside the GB300 hot path")


def _per_batch(x, B: int, shape_tail: tuple) -> np.ndarray:
    a = np.asarray(x, F32)
    return np.broadcast_to(a, (B, *shape_tail)).astype(F32)


def _descs(state: State, system) -> list:
    B, N, d = state.batch_size, state.N, state.dim
    dom = _domain_key(system)
    box = _per_batch(system.domain.box_size, B, (d,))
    anc = _per_batch(system.domain.anchor, B, (d,))
    grav = _per_batch(system.force_manager.gravity, B, (d,))
    dt = _per_batch(system.dt, B, ())
    e = _per_batch(getattr(system.domain, "restitution_coefficient", 1.0), B, ())
    coll = system.collider
    cell = _per_batch(getattr(coll, "cell_size", None) if getattr(coll, "cell_size", None) is not None else 1.0, B, ())
    sr = int(coll.search_range) if hasattr(coll, "search_range") and getattr(coll, "neighbor_mask", None) is not None else 1
    out = []
    for b in range(B):
        out.append(dict(n=N, domain=dom, linear=system.linear_integrator.type_name,
                        rotation=system.rotation_integrator.type_name, dt=float(dt[b]), box_size=box[b],
                        anchor=anc[b], restitution=float(e[b]), gravity=grav[b], cell_size=float(cell[b]),
                        search_range=sr))
    return out


def _bond_width(state: State) -> int:
    if state.bond_id.size == 0 or not np.any(state.bond_id >= 0):
        return 0
    return int(state.bond_id.shape[-1])


def _skin(state: State, system) -> float:
    from .autotune import default_skin

    s = getattr(system.collider, "skin", None)
    if s is None:
        s = default_skin(float(np.max(state.rad)) if state.rad.size else 1.0)
    return float(s)


def engine_for(state: State, system) -> Engine:
    """Cached engine handle for this static configuration."""
    _check_supported(state, system)
    descs = _descs(state, system)
    young = np.asarray(system.mat_table.young_eff, F32)
    W = _bond_width(state)
    skin = _skin(state, system)
    # a NeighborList collider's max_neighbors is the initial list capacity
    cap = getattr(system.collider, "max_neighbors", None)
    nl = int(cap) if cap else True
    key = (state.dim, W, bool(system.interact_same_bond_id), round(skin, 7), nl, young.tobytes(),
           tuple((d["n"], d["domain"], d["linear"], d["rotation"], d["dt"], tuple(map(float, d["box_size"])),
                  tuple(map(float, d["anchor"])), d["restitution"], tuple(map(float, d["gravity"])),
                  d["cell_size"], d["search_range"]) for d in descs))
    eng = _CACHE.get(key)
    if eng is None:
        eng = Engine(state.dim, descs, young, skin=skin, bond_width=W,
                     interact_same_bond_id=bool(system.interact_same_bond_id), neighbor_list=nl)
        _CACHE[key] = eng
        while len(_CACHE) > _CACHE_MAX:
            _, old = _CACHE.popitem(last=False)
            old.close()
    else:
        _CACHE.move_to_end(key)
    return eng


def clear_cache() -> None:
    while _CACHE:
        _, e = _CACHE.popitem()
        e.close()


def _flat(a: np.ndarray, P: int, tail: tuple) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a).reshape((P, *tail)))


def upload(eng: Engine, state: State) -> None:
    B, N, d = state.batch_size, state.N, state.dim
    P = B * N
    ad = 3 if d == 3 else 1
    W = eng.bond_width
    eng.upload(pos=_flat(state.pos_c, P, (d,)), rad=_flat(state.rad, P, ()), mass=_flat(state.mass, P, ()),
               vel=_flat(state.vel, P, (d,)), force=_flat(state.force, P, (d,)),
               q=_flat(state.q.as_array(), P, (4,)), ang_vel=_flat(state.ang_vel, P, (ad,)),
               torque=_flat(state.torque, P, (ad,)), inertia=_flat(state.inertia, P, (ad,)),
               mat_id=_flat(state.mat_id, P, ()), fixed=_flat(state.fixed, P, ()),
               bond_id=None if W == 0 else _bond_global(state, W))


def _bond_global(state: State, W: int) -> np.ndarray:
    """Per-system bond indices shifted to global particle indices."""
    B, N = state.batch_size, state.N
    bond = np.asarray(state.bond_id, np.int64).reshape(B, N, -1)[..., :W]
    off = (np.arange(B) * N)[:, None, None]
    return np.where(bond >= 0, bond + off, -1).reshape(B * N, W).astype(np.int32)


def download(eng: Engine, state: State) -> State:
    out = eng.download()
    st = state.copy()
    shp = state.pos_c.shape
    st.pos_c = out["pos_c"].reshape(shp)
    st.vel = out["vel"].reshape(shp)
    st.force = out["force"].reshape(shp)
    st.q = Quaternion.from_array(out["q"].reshape((*shp[:-1], 4)))
    st.ang_vel = out["ang_vel"].reshape(state.ang_vel.shape)
    st.torque = out["torque"].reshape(state.torque.shape)
    return st


def _advance_system(system, eng: Engine, n: int, batched: bool, index: int = 0):
    """time += dt per step in float32 (system.py:62-66); free-domain frame from the device
    (all systems of the handle when ``batched``, else system ``index``)."""
    dt = np.asarray(system.dt, F32)
    t = np.asarray(system.time, F32).copy()
    for _ in range(n):
        t = (t + dt).astype(F32)
    sc = (np.asarray(system.step_count) + n).astype(np.int32)
    dom = system.domain
    if dom.type_name == "free" and n > 0:
        box, anc = eng.domain_state()
        if not batched:
            box, anc = box[index], anc[index]
        dom = dataclasses.replace(dom, box_size=box.astype(F32), anchor=anc.astype(F32),
                                  inv_box_size=(F32(1.0) / box).astype(F32))
    return dataclasses.replace(system, time=t if t.ndim else F32(t), step_count=sc, domain=dom)


def step(state: State, system, n: int):
    if n < 0:
        raise ValueError("n must be >= 0")
    eng = engine_for(state, system)
    upload(eng, state)
    eng.step(n)
    return download(eng, state), _advance_system(system, eng, n, state.batch_size > 1 and state.pos_c.ndim == 3)


def rollout(state: State, system, strides: np.ndarray, save_fn: Callable):
    from .system import System

    eng = engine_for(state, system)
    upload(eng, state)
    frames = []
    st, sy = state, system
    batched = state.batch_size > 1 and state.pos_c.ndim == 3
    for k in strides:
        k = int(k)
        if k < 0:
            raise ValueError("strides must be >= 0")
        if k > 0:
            eng.step(k)
            st = download(eng, state)
            sy = _advance_system(sy, eng, k, batched)
        frames.append(save_fn(st, sy))
    traj = _stack_frames(frames)
    return st, sy, traj


def _stack_frames(frames):
    from .system import _tree_stack

    f0 = frames[0]
    if isinstance(f0, tuple):
        return tuple(_stack_frames([f[i] for f in frames]) for i in range(len(f0)))
    if isinstance(f0, State):
        return State.stack(frames)
    return _tree_stack(frames)


def compute_force(state: State, system):
    """Contact forces only (``cell_list.py:434-464``): no gravity, no integration."""
    eng = engine_for(state, system)
    upload(eng, state)
    eng.compute_force()
    st = download(eng, state)
    return st, system


def energies(state: State, system) -> np.ndarray:
    """``(pe_collider, pe_gravity, ke_trans, ke_rot)``, per batch member when batched."""
    eng = engine_for(state, system)
    upload(eng, state)
    e = eng.energy(per_system=True)
    return e if (state.batch_size > 1 and state.pos_c.ndim == 3) else e[0]


def neighbor_list(state: State, system, cutoff: float, max_neighbors: int):
    eng = engine_for(state, system)
    upload(eng, state)
    nl, ovf = eng.neighbor_list(cutoff, max_neighbors)
    if state.pos_c.ndim == 3:
        B, N = state.batch_size, state.N
        nl = nl.reshape(B, N, -1)
        off = (np.arange(B) * N)[:, None, None]
        nl = np.where(nl >= 0, nl - off, -1)
    return nl, ovf


def contacts(state: State, system) -> np.ndarray:
    eng = engine_for(state, system)
    upload(eng, state)
    return eng.contacts()
