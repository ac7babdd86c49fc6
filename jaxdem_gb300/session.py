"""Bridge between the host mirror (State/System) and the device engine.

A ``System`` plus a ``State`` (optionally batched along a leading axis, one
device system per batch member) map onto one engine handle
(``include/jdem_gb300.h``).  Handles are cached by their static
configuration, so repeated ``System.step`` calls reuse device memory and
captured CUDA graphs; each call uploads the caller's state, runs, and reads
the result back (the functional contract of the reference API).

Configurations outside the GB300 hot path raise ``NotImplementedError``:
facets, bonded force models, force models other than ``spring``, ``hertz``
and ``cundallstrack``, user force functions, pending external forces and
user pre/post-step actions.
"""

from __future__ import annotations

import collections
import dataclasses
from typing import Any, Callable, Optional

import numpy as np

from ._lib import DOMAIN, LINEAR, ROTATION, Engine, JdemError, load
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
    if system.force_model.type_name not in ("spring", "hertz", "cundallstrack"):
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
    if state.facet_id.size and np.any(state.facet_id != -1):
        raise NotImplementedError("facets are outside the GB300 hot path")


def _has_clumps(state: State) -> bool:
    """Rigid clumps: a body-frame offset, or a clump id shared by several spheres."""
    N = state.N
    if N == 0:
        return False
    if np.any(state.pos_p != 0):
        return True
    cid = state.clump_id.reshape(-1, N)
    return bool(np.any(cid != np.arange(N)))


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


def pair_law(system) -> tuple:
    """The force law's name, its (M, M) float32 pair constant (``young_eff`` for the
    spring, (4/3) E* for Hertz, the damping ratio for Cundall-Strack) and the
    per-material (M, 4) properties Cundall-Strack also needs (else None)."""
    law = system.force_model.type_name
    mt = system.mat_table
    if law == "hertz":
        from .forces import hertz_pair_constant

        return law, hertz_pair_constant(mt.young, mt.poisson), None
    if law == "cundallstrack":
        from .forces import cundall_strack_tables

        beta, props = cundall_strack_tables(mt.young, mt.poisson, mt.e, mt.mu, mt.mu_r)
        return law, beta, props
    return law, np.asarray(mt.young_eff, F32), None


def cached_engine(dim: int, descs: list, young: np.ndarray, *, skin: float, law: str = "spring",
                  props: Optional[np.ndarray] = None, bond_width: int = 0, interact_same_bond_id: bool = False,
                  neighbor_list=True) -> Engine:
    """Engine handle for this static configuration, reused across calls (device memory and
    captured CUDA graphs stay; each call uploads its own state)."""
    key = (dim, bond_width, bool(interact_same_bond_id), round(skin, 7), neighbor_list, law, young.tobytes(),
           None if props is None else props.tobytes(),
           tuple((d["n"], d["domain"], d["linear"], d["rotation"], d["dt"], tuple(map(float, d["box_size"])),
                  tuple(map(float, d["anchor"])), d["restitution"], tuple(map(float, d["gravity"])),
                  d["cell_size"], d["search_range"]) for d in descs))
    eng = _CACHE.get(key)
    if eng is None:
        eng = Engine(dim, descs, young, skin=skin, bond_width=bond_width,
                     interact_same_bond_id=bool(interact_same_bond_id), neighbor_list=neighbor_list, force_law=law,
                     material_props=props)
        _CACHE[key] = eng
        while len(_CACHE) > _CACHE_MAX:
            _, old = _CACHE.popitem(last=False)
            old.close()
    else:
        _CACHE.move_to_end(key)
    return eng


def engine_for(state: State, system) -> Engine:
    """Cached engine handle for this static configuration."""
    _check_supported(state, system)
    descs = _descs(state, system)
    law, young, props = pair_law(system)
    # a NeighborList collider's max_neighbors is the initial list capacity
    cap = getattr(system.collider, "max_neighbors", None)
    return cached_engine(state.dim, descs, young, skin=_skin(state, system), law=law, props=props,
                         bond_width=_bond_width(state), interact_same_bond_id=bool(system.interact_same_bond_id),
                         neighbor_list=int(cap) if cap else True)


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
               bond_id=None if W == 0 else _bond_global(state, W),
               pos_p=_flat(state.pos_p, P, (d,)) if _has_clumps(state) else None,
               clump_id=_flat(state.clump_id, P, ()) if _has_clumps(state) else None)


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


def _rotation_static(state: State) -> bool:
    """Identity orientations with zero angular velocity and torque: the engine leaves
    q, ang_vel and torque untouched (the spiral integrators keep them fixed)."""
    q = state.q
    return (bool(np.all(q.w == 1)) and not np.any(q.xyz) and not np.any(state.ang_vel)
            and not np.any(state.torque))


def _frame_times(system, strides: np.ndarray, batched: bool):
    """Per-frame ``time`` and ``step_count`` (float32 ``time += dt`` per step,
    system.py:62-66), accumulated in float32 step by step."""
    dt = np.asarray(system.dt, F32)
    t0 = np.asarray(system.time, F32)
    total = int(strides.sum())
    steps = np.cumsum(strides)
    if total:
        inc = np.broadcast_to(dt, (total, *dt.shape))
        acc = np.cumsum(np.concatenate([t0[None], inc], 0), axis=0, dtype=F32)
        times = acc[steps]
    else:
        times = np.broadcast_to(t0, (len(strides), *t0.shape)).copy()
    counts = (np.asarray(system.step_count)[None] + steps.reshape((-1,) + (1,) * np.ndim(system.step_count)))
    return times.astype(F32), counts.astype(np.int32)


def rollout(state: State, system, strides: np.ndarray, save_fn: Callable):
    """``System.trajectory_rollout`` on the device: frames are unpacked into a device
    ring after their strides and streamed to the host on a copy stream while the
    next stride runs (``jdem_rollout``)."""
    from .system import _save_state_system

    strides = np.asarray(strides, np.int64).reshape(-1)
    if np.any(strides < 0):
        raise ValueError("strides must be >= 0")
    T = len(strides)
    eng = engine_for(state, system)
    upload(eng, state)
    batched = state.batch_size > 1 and state.pos_c.ndim == 3
    # Cundall-Strack contacts and rigid clumps exert torques: the rotational state moves
    rot_static = (_rotation_static(state) and system.force_model.type_name != "cundallstrack"
                  and not _has_clumps(state))
    fields = ("pos_c", "vel", "force") if rot_static else Engine.FRAME_FIELDS
    free = system.domain.type_name == "free"
    fr = eng.rollout(strides, fields=fields, boxes=free)
    shp = state.pos_c.shape
    frames = {k: fr[k].reshape((T, *shp)) for k in ("pos_c", "vel", "force")}
    if rot_static:
        qa = state.q.as_array()
        frames["q"] = np.broadcast_to(qa, (T, *qa.shape))
        frames["ang_vel"] = np.broadcast_to(state.ang_vel, (T, *state.ang_vel.shape))
        frames["torque"] = np.broadcast_to(state.torque, (T, *state.torque.shape))
    else:
        frames["q"] = fr["q"].reshape((T, *shp[:-1], 4))
        frames["ang_vel"] = fr["ang_vel"].reshape((T, *state.ang_vel.shape))
        frames["torque"] = fr["torque"].reshape((T, *state.torque.shape))
    times, counts = _frame_times(system, strides, batched)
    boxes = anchors = None
    if free:
        boxes, anchors = fr["box"], fr["anchor"]
        if not batched:
            boxes, anchors = boxes[:, 0], anchors[:, 0]

    def frame_system(t: int):
        sy = dataclasses.replace(system, time=times[t] if times[t].ndim else F32(times[t]),
                                 step_count=counts[t] if counts[t].ndim else np.int32(counts[t]))
        if free:
            box = boxes[t].astype(F32)
            sy = dataclasses.replace(sy, domain=dataclasses.replace(
                system.domain, box_size=box, anchor=anchors[t].astype(F32), inv_box_size=(F32(1.0) / box).astype(F32)))
        return sy

    def frame_state(t: int, copy: bool = False) -> State:
        pick = (lambda a: np.array(a[t])) if copy else (lambda a: a[t])
        st = dataclasses.replace(state, pos_c=pick(frames["pos_c"]), vel=pick(frames["vel"]),
                                 force=pick(frames["force"]), q=Quaternion.from_array(frames["q"][t]),
                                 ang_vel=pick(frames["ang_vel"]), torque=pick(frames["torque"]))
        return st

    if T == 0:
        # a scan of length 0: every saved leaf gets an empty leading frame axis
        return state, system, _empty_frames(_stack_frames([save_fn(state, system)]))
    final_state, final_system = frame_state(T - 1, copy=True), frame_system(T - 1)
    if save_fn is _save_state_system:
        # the default save_fn stacks (state, system): build the stacked pytrees
        # from the frame arrays; static fields are read-only broadcasts
        kw = {}
        for f in dataclasses.fields(state):
            v = getattr(state, f.name)
            if f.name in frames and f.name != "q":
                kw[f.name] = frames[f.name]
            elif f.name == "q":
                qa = frames["q"]
                kw[f.name] = Quaternion(qa[..., 0:1], qa[..., 1:])
            else:
                kw[f.name] = np.broadcast_to(v, (T, *np.shape(v)))
        traj = (State(**kw), _stack_frames([frame_system(t) for t in range(T)]))
        return final_state, final_system, traj
    return final_state, final_system, _stack_frames([save_fn(frame_state(t), frame_system(t)) for t in range(T)])


def _empty_frames(tree):
    if isinstance(tree, tuple):
        return tuple(_empty_frames(x) for x in tree)
    if isinstance(tree, Quaternion):
        return Quaternion(tree.w[:0], tree.xyz[:0])
    if dataclasses.is_dataclass(tree):
        kw = {}
        for f in dataclasses.fields(tree):
            v = getattr(tree, f.name)
            kw[f.name] = _empty_frames(v) if isinstance(v, (np.ndarray, tuple, Quaternion)) or (
                dataclasses.is_dataclass(v) and not callable(v)) else v
        return dataclasses.replace(tree, **kw)
    if isinstance(tree, np.ndarray):
        return tree[:0]
    return tree


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



class _DeviceArrays:
    """Torch tensors on the current device for the stage entry points: one (B, N, ...)
    float32 (or given dtype) tensor per state field, and the current stream."""

    def __init__(self, state: State):
        import torch

        self.torch = torch
        self.dev = torch.device("cuda", torch.cuda.current_device())
        self.B, self.N, self.d = state.batch_size, state.N, state.dim
        self.stream = torch.cuda.current_stream(self.dev).cuda_stream

    def put(self, a, tail, dtype=np.float32):
        arr = np.ascontiguousarray(np.asarray(a, dtype).reshape((self.B, self.N) + tail))
        return self.torch.from_numpy(arr).to(self.dev)

    def finish(self):
        self.torch.cuda.current_stream(self.dev).synchronize()


def _per_system(x, B: int, tail: tuple) -> np.ndarray:
    return np.broadcast_to(np.asarray(x, np.float32), (B, *tail) if tail else (B,)).reshape((B, *tail))


def domain_apply(state: State, system):
    """``Domain.apply`` (first stage of ``_step_once``, ``system.py:60-82``) on the GPU
    (``jdem_domain_apply``): reflecting walls move and kick spheres, the free domain's box
    follows the particles, the periodic domain does nothing.  Returns a new state and
    system (the reference's functional contract)."""
    dom = system.domain
    key = dom.type_name
    if key not in DOMAIN:
        raise NotImplementedError(f"domain {key!r} is outside the GB300 hot path")
    st = state.copy()
    if key == "periodic" or state.N == 0:
        return st, system
    if _has_clumps(state):
        raise NotImplementedError("Domain.apply of rigid clumps runs inside System.step")
    lib = load()
    A = _DeviceArrays(state)
    B, N, d = A.B, A.N, A.d
    box = _per_system(dom.box_size, B, (d,))
    anc = _per_system(dom.anchor, B, (d,))
    dts = _per_system(system.dt, B, ())
    rest = _per_system(getattr(dom, "restitution_coefficient", 1.0), B, ())
    pos, vel, frc = A.put(st.pos_c, (d,)), A.put(st.vel, (d,)), A.put(st.force, (d,))
    rad, mass, fixed = A.put(st.rad, ()), A.put(st.mass, ()), A.put(st.fixed, (), np.uint8)
    q = A.put(st.q.as_array(), (4,))
    box_out, anc_out = np.zeros((B, d), F32), np.zeros((B, d), F32)
    for b in range(B):
        bx, an = np.ascontiguousarray(box[b]), np.ascontiguousarray(anc[b])
        rc = lib.jdem_domain_apply(d, N, DOMAIN[key], float(dts[b]), float(rest[b]), bx.ctypes.data, an.ctypes.data,
                                   pos[b].data_ptr(), vel[b].data_ptr(), frc[b].data_ptr(), rad[b].data_ptr(),
                                   mass[b].data_ptr(), fixed[b].data_ptr(), None, q[b].data_ptr(),
                                   box_out[b].ctypes.data, anc_out[b].ctypes.data, A.stream)
        if rc != 0:
            raise JdemError(rc, "jdem_domain_apply failed")
    A.finish()
    if key == "free":
        shp = np.shape(dom.box_size)
        nb, na = box_out.reshape(shp), anc_out.reshape(shp)
        return st, dataclasses.replace(system, domain=dataclasses.replace(dom, box_size=nb, anchor=na))
    shp = state.pos_c.shape
    st.pos_c = pos.cpu().numpy().reshape(shp)
    st.vel = vel.cpu().numpy().reshape(shp)
    st.q = Quaternion.from_array(q.cpu().numpy().reshape((*shp[:-1], 4)))
    return st, system


def force_manager_apply(state: State, system):
    """``ForceManager.apply`` (``force_manager.py:338-425``) for spheres on the GPU
    (``jdem_force_manager_apply``): the external buffers and gravity join the contact
    force and torque, and the returned system's external buffers are cleared."""
    fm = system.force_manager
    if getattr(fm, "force_functions", ()):
        raise NotImplementedError("user force functions are outside the GB300 hot path")
    st = state.copy()
    if state.N == 0:
        return st, system
    if _has_clumps(state):
        raise NotImplementedError("ForceManager.apply of rigid clumps runs inside System.step")
    lib = load()
    A = _DeviceArrays(state)
    B, N, d = A.B, A.N, A.d
    ad = 3 if d == 3 else 1
    grav = _per_system(fm.gravity, B, (d,))
    frc, tq, mass = A.put(st.force, (d,)), A.put(st.torque, (ad,)), A.put(st.mass, ())
    ef, efc, et = A.put(fm.external_force, (d,)), A.put(fm.external_force_com, (d,)), A.put(fm.external_torque, (ad,))
    for b in range(B):
        g = np.ascontiguousarray(grav[b])
        rc = lib.jdem_force_manager_apply(d, N, g.ctypes.data, frc[b].data_ptr(), tq[b].data_ptr(), ef[b].data_ptr(),
                                          efc[b].data_ptr(), et[b].data_ptr(), mass[b].data_ptr(), A.stream)
        if rc != 0:
            raise JdemError(rc, "jdem_force_manager_apply failed")
    A.finish()
    shp = state.pos_c.shape
    st.force = frc.cpu().numpy().reshape(shp)
    st.torque = tq.cpu().numpy().reshape(state.torque.shape)
    nfm = dataclasses.replace(fm, external_force=np.zeros_like(fm.external_force),
                              external_force_com=np.zeros_like(fm.external_force_com),
                              external_torque=np.zeros_like(fm.external_torque))
    return st, dataclasses.replace(system, force_manager=nfm)


def integrate_stage(state: State, system, linear: str, rotation: str, stage: int):
    """One integrator stage on the GPU (``jdem_integrate``): ``step_before_force``
    (stage 0) or ``step_after_force`` (stage 1) of the linear integrator ``linear``
    and the rotation integrator ``rotation`` (either may be ``""``), as the split
    factory types call them (``integrators/__init__.py:51-91``).  Returns a new state
    and the system, the reference's functional contract.  Batched states take each
    system's own ``dt``.  Device buffers are torch tensors on the current device and
    the work is queued on torch's current stream."""
    lin, rot = LINEAR[linear], ROTATION[rotation]
    st = state.copy()
    if (lin == 0 and rot == 0) or (lin == LINEAR["euler"] and rot == 0 and stage == 0):
        return st, system
    lib = load()
    A = _DeviceArrays(state)
    B, N, d = A.B, A.N, A.d
    ad = 3 if d == 3 else 1
    dts = _per_system(system.dt, B, ())
    pos, vel, frc = A.put(st.pos_c, (d,)), A.put(st.vel, (d,)), A.put(st.force, (d,))
    mass, fixed = A.put(st.mass, ()), A.put(st.fixed, (), np.uint8)
    q, w = A.put(st.q.as_array(), (4,)), A.put(st.ang_vel, (ad,))
    tq, inertia = A.put(st.torque, (ad,)), A.put(st.inertia, (ad,))
    stream = A.stream
    for b in range(B):
        rc = lib.jdem_integrate(d, N, lin, rot, int(stage), float(dts[b]), pos[b].data_ptr(), vel[b].data_ptr(),
                                frc[b].data_ptr(), mass[b].data_ptr(), fixed[b].data_ptr(), q[b].data_ptr(),
                                w[b].data_ptr(), tq[b].data_ptr(), inertia[b].data_ptr(), stream)
        if rc != 0:
            raise JdemError(rc, "jdem_integrate failed")
    A.finish()
    shp = state.pos_c.shape
    st.pos_c = pos.cpu().numpy().reshape(shp)
    st.vel = vel.cpu().numpy().reshape(shp)
    st.q = Quaternion.from_array(q.cpu().numpy().reshape((*shp[:-1], 4)))
    st.ang_vel = w.cpu().numpy().reshape(state.ang_vel.shape)
    return st, system
