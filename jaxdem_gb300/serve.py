"""Serving: rollout requests of different size, dimension and length, admitted
into a continuously batched device handle (``jdem_serve_*`` in
``include/jdem_gb300.h``).

A request is ``System.step(state, system, n=steps)`` on one independent
sphere system: its own domain, integrators (rotation included), dt, material
ids and rotational state, under the server's force law (spring, Hertz or
Cundall-Strack) and material table.  ``Server`` wraps one dimension; ``run_stream`` replays a
timed arrival stream on a 2D and a 3D server at once and reports latency
percentiles and throughput; ``run_one_at_a_time`` serves the same stream with
the plain kernel, one request after another, for comparison.
"""

from __future__ import annotations

import ctypes as C
import threading
import time
from typing import Optional, Sequence

import numpy as np

from ._lib import DOMAIN, FORCE_LAW, LINEAR, ROTATION, Engine, HostState, JdemError, SystemDesc, load
from .autotune import default_skin
from .workloads import K_SPRING, Request as StreamRequest, Workload

F32 = np.float32
STATES = {0: "pending", 1: "active", 2: "done", 3: "cancelled", 4: "failed"}


class ServeConfig(C.Structure):
    _fields_ = [("dim", C.c_int32), ("device", C.c_int32), ("max_active", C.c_int32), ("chunk_steps", C.c_int32),
                ("target_particles", C.c_int64), ("hbm_budget_bytes", C.c_double), ("skin", C.c_float),
                ("young", C.c_float), ("force_law", C.c_int32), ("n_materials", C.c_int32),
                ("young_eff", C.c_void_p), ("material_props", C.c_void_p)]


class RequestStruct(C.Structure):
    _fields_ = [("system", SystemDesc), ("steps", C.c_int64), ("pos", C.c_void_p), ("vel", C.c_void_p),
                ("rad", C.c_void_p), ("mass", C.c_void_p), ("mat_id", C.c_void_p), ("q", C.c_void_p),
                ("ang_vel", C.c_void_p)]


class RequestInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("n", C.c_int64), ("steps", C.c_int64),
                ("submit_s", C.c_double), ("admit_s", C.c_double), ("done_s", C.c_double)]


class ServeStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("submitted", "completed", "epochs", "repacks", "particle_steps",
                                          "max_active", "failures", "pending", "active", "bytes_in_use")]


_PROTOS = [
    ("jdem_serve_create", [C.POINTER(ServeConfig), C.POINTER(C.c_void_p)], C.c_int),
    ("jdem_serve_submit", [C.c_void_p, C.POINTER(RequestStruct), C.POINTER(C.c_int64)], C.c_int),
    ("jdem_serve_cancel", [C.c_void_p, C.c_int64], C.c_int),
    ("jdem_serve_poll", [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)], C.c_int),
    ("jdem_serve_result", [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(RequestInfo)],
     C.c_int),
    ("jdem_serve_result_state", [C.c_void_p, C.c_int64, C.c_void_p, C.POINTER(RequestInfo)], C.c_int),
    ("jdem_serve_release", [C.c_void_p, C.c_int64], C.c_int),
    ("jdem_serve_drain", [C.c_void_p, C.c_double], C.c_int),
    ("jdem_serve_stats", [C.c_void_p, C.POINTER(ServeStats)], C.c_int),
    ("jdem_serve_last_error", [C.c_void_p], C.c_char_p),
    ("jdem_serve_destroy", [C.c_void_p], C.c_int),
]


def _lib():
    lib = load()
    if not getattr(lib, "_serve_bound", False):
        for name, argt, rest in _PROTOS:
            fn = getattr(lib, name)
            fn.argtypes = argt
            fn.restype = rest
        lib._serve_bound = True
    return lib


def _desc(w: Workload, rotation: str = "") -> SystemDesc:
    d = SystemDesc()
    d.n = w.N
    d.domain = DOMAIN[w.domain]
    d.linear_integrator = LINEAR["verlet"]
    d.rotation_integrator = ROTATION[rotation]
    d.dt = float(w.dt)
    for a in range(3):
        d.box_size[a] = float(w.box_size[a]) if a < w.dim else 1.0
        d.anchor[a] = float(w.anchor[a]) if a < w.dim else 0.0
        d.gravity[a] = float(w.gravity[a]) if a < w.dim else 0.0
    d.restitution = float(w.restitution)
    d.cell_size = 2.0 * float(w.rad.max()) if w.N else 1.0
    d.search_range = 1
    return d


class Server:
    """Continuous-batching server for one dimension."""

    def __init__(self, dim: int, *, max_active: int = 1024, chunk_steps: int = 50,
                 target_particles: int = 4 << 20, hbm_budget_gb: float = 150.0, skin: Optional[float] = None,
                 rmax: float = 0.6, young: float = K_SPRING, device: int = 0, force_law: str = "spring",
                 young_eff: Optional[np.ndarray] = None, material_props: Optional[np.ndarray] = None):
        """``young_eff`` (M, M): the force law's pair constant per material pair (spring k,
        Hertz (4/3) E*, Cundall-Strack beta); None: one material of stiffness ``young``.
        ``material_props`` (M, 4): Cundall-Strack's (young, shear modulus, mu, mu_r) per
        material (both tables required for ``force_law="cundallstrack"``)."""
        self.lib = _lib()
        self.dim = dim
        if force_law not in FORCE_LAW:
            raise ValueError(f"unknown force law '{force_law}'")
        if force_law == "cundallstrack" and (young_eff is None or material_props is None):
            raise ValueError("Cundall-Strack needs young_eff (beta) and material_props")
        table = None if young_eff is None else np.ascontiguousarray(young_eff, F32)
        props = None if material_props is None else np.ascontiguousarray(material_props, F32).reshape(-1, 4)
        if props is not None and table is not None and props.shape[0] != table.shape[0]:
            raise ValueError("material_props must have one row per material")
        cfg = ServeConfig(dim=dim, device=device, max_active=max_active, chunk_steps=chunk_steps,
                          target_particles=int(target_particles), hbm_budget_bytes=hbm_budget_gb * 1e9,
                          skin=float(default_skin(rmax) if skin is None else skin), young=float(young),
                          force_law=FORCE_LAW[force_law], n_materials=0 if table is None else table.shape[0],
                          young_eff=None if table is None else table.ctypes.data,
                          material_props=None if props is None or force_law != "cundallstrack" else props.ctypes.data)
        h = C.c_void_p()
        rc = self.lib.jdem_serve_create(C.byref(cfg), C.byref(h))
        if rc:
            raise JdemError(rc, "jdem_serve_create failed")
        self.h = h

    def _check(self, rc: int) -> None:
        if rc:
            msg = self.lib.jdem_serve_last_error(self.h)
            raise JdemError(rc, msg.decode() if msg else "")

    def submit(self, w: Workload, steps: Optional[int] = None, *, mat_id=None, q=None, ang_vel=None,
               rotation: str = "") -> int:
        """Queue ``System.step(state, system, n=steps)``; ``rotation`` names the request's
        rotation integrator ("", "verletspiral", "spiral"), ``q`` / ``ang_vel`` its rotational
        state (identity / zero when None)."""
        if w.dim != self.dim:
            raise ValueError("request dimension does not match the server")
        arrs = [np.ascontiguousarray(a, F32) for a in (w.pos, w.vel, w.rad, w.mass)]
        ad = 3 if self.dim == 3 else 1
        mat = None if mat_id is None else np.ascontiguousarray(mat_id, np.int32).reshape(w.N)
        qa = None if q is None else np.ascontiguousarray(q, F32).reshape(w.N, 4)
        wa = None if ang_vel is None else np.ascontiguousarray(ang_vel, F32).reshape(w.N, ad)
        req = RequestStruct(system=_desc(w, rotation), steps=int(w.steps if steps is None else steps),
                            pos=arrs[0].ctypes.data, vel=arrs[1].ctypes.data, rad=arrs[2].ctypes.data,
                            mass=arrs[3].ctypes.data, mat_id=None if mat is None else mat.ctypes.data,
                            q=None if qa is None else qa.ctypes.data, ang_vel=None if wa is None else wa.ctypes.data)
        rid = C.c_int64()
        self._check(self.lib.jdem_serve_submit(self.h, C.byref(req), C.byref(rid)))
        return int(rid.value)

    def cancel(self, rid: int) -> None:
        self._check(self.lib.jdem_serve_cancel(self.h, int(rid)))

    def poll(self) -> list:
        ids = np.zeros(4096, np.int64)
        n = C.c_int32()
        self._check(self.lib.jdem_serve_poll(self.h, ids.ctypes.data, ids.size, C.byref(n)))
        return ids[: n.value].tolist()

    def info(self, rid: int) -> dict:
        inf = RequestInfo()
        self.lib.jdem_serve_result(self.h, int(rid), None, None, None, C.byref(inf))
        return {"state": STATES.get(inf.state, inf.state), "status": inf.status, "n": inf.n, "steps": inf.steps,
                "submit_s": inf.submit_s, "admit_s": inf.admit_s, "done_s": inf.done_s}

    def result(self, rid: int) -> dict:
        """Final pos_c, vel, force, q and ang_vel of a done request, and its timings."""
        inf = RequestInfo()
        self.lib.jdem_serve_result(self.h, int(rid), None, None, None, C.byref(inf))
        n = int(inf.n)
        ad = 3 if self.dim == 3 else 1
        out = {k: np.empty((n, self.dim), F32) for k in ("pos_c", "vel", "force")}
        out["q"] = np.empty((n, 4), F32)
        out["ang_vel"] = np.empty((n, ad), F32)
        hs = HostState()
        for k in ("pos_c", "vel", "force", "q", "ang_vel"):
            setattr(hs, k, out[k].ctypes.data)
        self._check(self.lib.jdem_serve_result_state(self.h, int(rid), C.byref(hs), C.byref(inf)))
        out["info"] = self.info(rid)
        return out

    def release(self, rid: int) -> None:
        self._check(self.lib.jdem_serve_release(self.h, int(rid)))

    def drain(self, timeout: float = 0.0) -> None:
        self._check(self.lib.jdem_serve_drain(self.h, float(timeout)))

    def stats(self) -> dict:
        st = ServeStats()
        self._check(self.lib.jdem_serve_stats(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServeStats._fields_}

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.jdem_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _percentiles(x) -> dict:
    x = np.asarray(x, np.float64)
    if x.size == 0:
        return {"p50": None, "p99": None, "mean": None}
    return {"p50": float(np.percentile(x, 50)), "p99": float(np.percentile(x, 99)), "mean": float(x.mean())}


def run_stream(requests: Sequence[StreamRequest], *, time_scale: float = 1.0, max_active: int = 1024,
               target_particles: int = 4 << 20, chunk_steps: int = 50, device: int = 0,
               timeout: float = 600.0) -> dict:
    """Replay an arrival stream on a 2D and a 3D server (continuous batching)."""
    work = [(r, r.workload()) for r in requests]  # generated before the clock starts
    servers = {d: Server(d, max_active=max_active, target_particles=target_particles, chunk_steps=chunk_steps,
                         device=device) for d in (2, 3)}
    ids = {}
    t0 = time.perf_counter()

    def feed():
        for r, w in work:
            delay = t0 + r.arrival * time_scale - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            ids[(w.dim, servers[w.dim].submit(w))] = r

    th = threading.Thread(target=feed)
    th.start()
    th.join()
    lat, waits, psteps = [], [], 0
    for d, s in servers.items():
        s.drain(timeout)
    t_end = time.perf_counter()
    first_submit, last_done = None, None
    for (d, rid), r in ids.items():
        inf = servers[d].info(rid)
        if inf["state"] != "done":
            continue
        lat.append(inf["done_s"] - inf["submit_s"])
        waits.append(inf["admit_s"] - inf["submit_s"])
        psteps += inf["n"] * inf["steps"]
        first_submit = inf["submit_s"] if first_submit is None else min(first_submit, inf["submit_s"])
        last_done = inf["done_s"] if last_done is None else max(last_done, inf["done_s"])
        servers[d].release(rid)
    stats = {d: s.stats() for d, s in servers.items()}
    for s in servers.values():
        s.close()
    makespan = (last_done - first_submit) if lat else float("nan")
    return {"completed": len(lat), "requests": len(requests), "particle_steps": psteps,
            "makespan_s": makespan, "throughput": psteps / makespan if lat else 0.0,
            "latency_s": _percentiles(lat), "queue_wait_s": _percentiles(waits), "wall_s": t_end - t0,
            "server_stats": {str(d): st for d, st in stats.items()}}


def run_one_at_a_time(requests: Sequence[StreamRequest], *, time_scale: float = 1.0, device: int = 0,
                      chunk_steps: int = 50, paced: bool = True) -> dict:
    """The plain kernel serving one request at a time, in arrival order (one handle per request).
    With ``paced`` False the requests run back to back (service times only)."""
    work = [(r, r.workload()) for r in requests]
    t0 = time.perf_counter()
    lat, psteps, service = [], 0, []
    busy = 0.0
    for r, w in work:
        arrive = t0 + r.arrival * time_scale
        now = time.perf_counter()
        if paced and now < arrive:
            time.sleep(arrive - now)
        a = time.perf_counter()
        eng = Engine(w.dim, [w.desc()], np.array([[K_SPRING]], F32), skin=default_skin(float(w.rad.max())),
                     chunk_steps=chunk_steps, device=device)
        try:
            eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
            eng.step(r.steps)
            eng.download()
        finally:
            eng.close()
        done = time.perf_counter()
        busy += done - a
        service.append(done - a)
        lat.append(done - arrive)
        psteps += w.N * r.steps
    makespan = time.perf_counter() - t0 - work[0][0].arrival * time_scale
    return {"completed": len(lat), "particle_steps": psteps, "makespan_s": makespan,
            "throughput": psteps / makespan, "busy_throughput": psteps / busy,
            "latency_s": _percentiles(lat) if paced else None, "service_s": service}


def fifo_model(window: Sequence[StreamRequest], timed: Sequence[StreamRequest], service_s: Sequence[float]) -> dict:
    """Latency of a one-at-a-time FIFO server over ``window``'s arrivals, with service
    times predicted per dimension as a + b * N * steps from the timed requests."""
    coef = {}
    for d in (2, 3):
        xs = np.array([r.N * r.steps for r in timed if r.dim == d], np.float64)
        ys = np.array([t for r, t in zip(timed, service_s) if r.dim == d], np.float64)
        if len(xs) >= 2:
            A = np.stack([np.ones_like(xs), xs], 1)
            a, b = np.linalg.lstsq(A, ys, rcond=None)[0]
            coef[d] = (max(float(a), 0.0), max(float(b), 0.0))
        else:
            rate = float(np.sum(xs) / max(np.sum(ys), 1e-12)) if len(xs) else 1e9
            coef[d] = (0.0, 1.0 / rate)
    free_at, lat = 0.0, []
    for r in window:
        a, b = coef[r.dim]
        start = max(free_at, r.arrival)
        free_at = start + a + b * r.N * r.steps
        lat.append(free_at - r.arrival)
    return {"latency_s": _percentiles(lat), "coef": {str(d): c for d, c in coef.items()}}
