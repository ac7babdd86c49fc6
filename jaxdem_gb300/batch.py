"""Batching layer: many independent systems of uneven size in one device handle.

The reference batches only systems of equal N, through ``jax.vmap``
(``system.py:743-744``), and its vmapped while-loops run to the worst
member's occupancy (``cell_list.py:357-365``).  Here every system keeps its
own segment of particles and of cells (segmented cell lists, per-system
offsets), and one launch of each kernel advances all of them; steps are
captured in CUDA graphs of ``chunk_steps`` steps.
"""

from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from . import autotune
from ._lib import Engine
from .state import Quaternion
from .workloads import K_SPRING, Workload

F32 = np.float32


class BatchedSystems:
    """Independent systems (same dimension) stepped together.

    ``workloads`` are :class:`jaxdem_gb300.workloads.Workload` records (or any
    object with ``pos, vel, rad, mass, dim, N`` and a ``desc()`` method).
    """

    def __init__(self, workloads: Sequence[Workload], young: float = K_SPRING, skin: Optional[float] = None,
                 chunk_steps: int = 50, device: int = 0, neighbor_list=True, **shapes):
        """``shapes`` are the engine's tunable shapes (``prune_skin``, ``brick_particles``,
        ``force_block``, ``small_lanes``; see ``autotune.tune_shapes``)."""
        if not workloads:
            raise ValueError("no systems")
        dims = {w.dim for w in workloads}
        if len(dims) != 1:
            raise ValueError("all systems of a batch must have the same dimension")
        self.dim = dims.pop()
        self.workloads = list(workloads)
        self.n = np.array([w.N for w in workloads], np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.n)])
        rmax = max(float(w.rad.max()) for w in workloads if w.N)
        self.skin = float(skin) if skin is not None else autotune.default_skin(rmax)
        self.engine = Engine(self.dim, [w.desc() for w in workloads], np.array([[young]], F32), skin=self.skin,
                             chunk_steps=chunk_steps, device=device, neighbor_list=neighbor_list, **shapes)

    def upload(self) -> None:
        cat = lambda k: np.concatenate([getattr(w, k) for w in self.workloads])  # noqa: E731
        self.engine.upload(pos=cat("pos"), rad=cat("rad"), mass=cat("mass"), vel=cat("vel"))

    def step(self, n: int) -> None:
        self.engine.step(n)

    def step_async(self, n: int) -> None:
        self.engine.step_async(n)

    def download(self) -> list:
        out = self.engine.download()
        res = []
        for s in range(len(self.workloads)):
            a, b = self.offsets[s], self.offsets[s + 1]
            res.append({k: v[a:b] for k, v in out.items()})
        return res

    def energies(self) -> np.ndarray:
        return self.engine.energy(per_system=True)

    def tune_key(self) -> str:
        return tune_key(self.workloads)

    @property
    def particles(self) -> int:
        return int(self.offsets[-1])

    def close(self) -> None:
        self.engine.close()


def tune_key(workloads: Sequence[Workload]) -> str:
    """Autotuner cache key of a batch: dimension, total particles, overall packing
    fraction and speed (``autotune.config_key``) plus the number of systems."""
    from .workloads import volume

    dim = workloads[0].dim
    n = sum(int(w.N) for w in workloads)
    vol = sum(float(np.prod(np.asarray(w.box_size, np.float64))) for w in workloads)
    occ = sum(float(volume(w.rad, w.dim).astype(np.float64).sum()) for w in workloads)
    v2 = sum(float((np.asarray(w.vel, np.float64) ** 2).sum()) for w in workloads)
    vrms = float(np.sqrt(v2 / max(1, n * dim)))
    return f"batch{len(workloads)}-" + autotune.config_key(dim, n, occ / max(vol, 1e-30), vrms, "periodic")


def step_many(states, systems, n: int):
    """``System.step`` over a list of (state, system) pairs of possibly different N,
    in one batched device handle per dimension; returns lists of states and systems.
    Handles are cached by the batch's static configuration (the systems' sizes,
    domains, integrators, force law and materials), so repeated calls on batches of
    the same shape reuse device memory and captured CUDA graphs."""
    from . import session
    from .state import State

    if len(states) != len(systems):
        raise ValueError("states and systems must have the same length")
    out_states, out_systems = [None] * len(states), [None] * len(states)
    by_dim: dict = {}
    for k, st in enumerate(states):
        by_dim.setdefault(st.dim, []).append(k)
    for dim, idx in by_dim.items():
        for k in idx:
            session._check_supported(states[k], systems[k])
        descs = [session._descs(states[k], systems[k])[0] for k in idx]
        law, young, props = session.pair_law(systems[idx[0]])
        for k in idx[1:]:
            lk, yk, pk = session.pair_law(systems[k])
            if lk != law or not np.array_equal(yk, young) or (props is not None and not np.array_equal(pk, props)):
                raise NotImplementedError("systems of one batch must share the force law and material table")
        skin = max(session._skin(states[k], systems[k]) for k in idx)
        eng = session.cached_engine(dim, descs, young, skin=skin, law=law, props=props)
        cat = lambda f: np.concatenate([np.asarray(f(states[k])) for k in idx])  # noqa: E731
        ad = 3 if dim == 3 else 1
        eng.upload(pos=cat(lambda s: s.pos_c), rad=cat(lambda s: s.rad), mass=cat(lambda s: s.mass),
                   vel=cat(lambda s: s.vel), force=cat(lambda s: s.force),
                   q=cat(lambda s: s.q.as_array()), ang_vel=cat(lambda s: s.ang_vel.reshape(-1, ad)),
                   torque=cat(lambda s: s.torque.reshape(-1, ad)),
                   inertia=cat(lambda s: s.inertia.reshape(-1, ad)), mat_id=cat(lambda s: s.mat_id),
                   fixed=cat(lambda s: s.fixed))
        eng.step(n)
        res = eng.download()
        off = 0
        for k in idx:
            st = states[k]
            N = st.N
            sub = State.copy(st)
            sub.pos_c = res["pos_c"][off:off + N].copy()
            sub.vel = res["vel"][off:off + N].copy()
            sub.force = res["force"][off:off + N].copy()
            sub.q = Quaternion.from_array(res["q"][off:off + N])
            sub.ang_vel = res["ang_vel"][off:off + N].reshape(st.ang_vel.shape)
            sub.torque = res["torque"][off:off + N].reshape(st.torque.shape)
            out_states[k] = sub
            out_systems[k] = session._advance_system(systems[k], eng, n, False, index=idx.index(k))
            off += N
    return out_states, out_systems
