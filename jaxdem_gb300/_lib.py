"""ctypes binding of ``libjdem_gb300.so`` (the C ABI in ``include/jdem_gb300.h``).

This is the only route from Python to the device: there is no CPU fallback.
Loading raises ``RuntimeError`` when the library has not been built, and every
failing call raises :class:`JdemError` carrying the library's message.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

# JDEM_LIBRARY names another build of the same library: the bounds-checked one
# (build.build(checked=True)) in the tests that run it
LIB_PATH = Path(os.environ.get("JDEM_LIBRARY") or Path(__file__).resolve().parent / "_lib" / "libjdem_gb300.so")

JDEM_OK = 0
STATUS_NAMES = {
    0: "ok",
    1: "bad argument",
    2: "capacity overflow",
    3: "hash overflow",
    4: "non-finite state",
    5: "out of device memory",
    6: "timeout",
    7: "unsupported configuration",
    8: "CUDA error",
    9: "not ready",
}

DOMAIN = {"free": 0, "periodic": 1, "reflect": 2}
LINEAR = {"": 0, "verlet": 1, "euler": 2}
ROTATION = {"": 0, "verletspiral": 1, "spiral": 2}
FORCE_LAW = {"spring": 0, "hertz": 1, "cundallstrack": 2}


class JdemError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{STATUS_NAMES.get(code, code)}] {msg}")
        self.code = code


class SystemDesc(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("domain", C.c_int32),
        ("linear_integrator", C.c_int32),
        ("rotation_integrator", C.c_int32),
        ("dt", C.c_float),
        ("box_size", C.c_float * 3),
        ("anchor", C.c_float * 3),
        ("restitution", C.c_float),
        ("gravity", C.c_float * 3),
        ("cell_size", C.c_float),
        ("search_range", C.c_int32),
    ]


class Config(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("n_systems", C.c_int32),
        ("systems", C.POINTER(SystemDesc)),
        ("skin", C.c_float),
        ("n_materials", C.c_int32),
        ("young_eff", C.POINTER(C.c_float)),
        ("bond_width", C.c_int32),
        ("interact_same_bond_id", C.c_int32),
        ("chunk_steps", C.c_int32),
        ("device", C.c_int32),
        ("neighbor_list", C.c_int32),
        ("graph_mode", C.c_int32),
        ("force_law", C.c_int32),
        ("material_props", C.POINTER(C.c_float)),
        ("prune_skin", C.c_float),
        ("brick_particles", C.c_int32),
        ("force_block", C.c_int32),
        ("small_lanes", C.c_int32),
    ]


class HostState(C.Structure):
    _fields_ = [
        ("pos_c", C.c_void_p),
        ("vel", C.c_void_p),
        ("force", C.c_void_p),
        ("q", C.c_void_p),
        ("ang_vel", C.c_void_p),
        ("torque", C.c_void_p),
        ("rad", C.c_void_p),
        ("mass", C.c_void_p),
        ("inertia", C.c_void_p),
        ("mat_id", C.c_void_p),
        ("fixed", C.c_void_p),
        ("bond_id", C.c_void_p),
        ("pos_p", C.c_void_p),
        ("clump_id", C.c_void_p),
    ]


class Frames(C.Structure):
    _fields_ = [
        ("pos_c", C.c_void_p),
        ("vel", C.c_void_p),
        ("force", C.c_void_p),
        ("q", C.c_void_p),
        ("ang_vel", C.c_void_p),
        ("torque", C.c_void_p),
        ("box", C.c_void_p),
        ("anchor", C.c_void_p),
        ("device_ptrs", C.c_int32),
        ("ring", C.c_int32),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("n_particles", C.c_int64),
        ("n_cells", C.c_int64),
        ("n_systems", C.c_int32),
        ("dim", C.c_int32),
        ("rebuilds", C.c_int64),
        ("steps", C.c_int64),
        ("device_status", C.c_uint32),
        ("graphs", C.c_int32),
        ("device_bytes", C.c_int64),
        ("list_regrowths", C.c_int64),
        ("list_capacity", C.c_int32),
        ("list_tiles", C.c_int32),
        ("many_step", C.c_int32),
        ("prunes", C.c_int32),
    ]


_LIB: Optional[C.CDLL] = None

# (name, argtypes, restype) of every exported entry point
_PROTOS = [
    ("jdem_abi_version", [], C.c_int),
    ("jdem_status_string", [C.c_int], C.c_char_p),
    ("jdem_create", [C.POINTER(Config), C.POINTER(C.c_void_p)], C.c_int),
    ("jdem_destroy", [C.c_void_p], C.c_int),
    ("jdem_last_error", [C.c_void_p], C.c_char_p),
    ("jdem_upload", [C.c_void_p, C.POINTER(HostState)], C.c_int),
    ("jdem_upload_device", [C.c_void_p, C.POINTER(HostState)], C.c_int),
    ("jdem_step", [C.c_void_p, C.c_int64], C.c_int),
    ("jdem_step_async", [C.c_void_p, C.c_int64], C.c_int),
    ("jdem_sync", [C.c_void_p], C.c_int),
    ("jdem_step_timed", [C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
    ("jdem_download", [C.c_void_p, C.POINTER(HostState)], C.c_int),
    ("jdem_download_device", [C.c_void_p, C.POINTER(HostState)], C.c_int),
    ("jdem_rollout", [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(Frames)], C.c_int),
    ("jdem_compute_force", [C.c_void_p], C.c_int),
    ("jdem_energy", [C.c_void_p, C.POINTER(C.c_double)], C.c_int),
    ("jdem_energy_per_system", [C.c_void_p, C.POINTER(C.c_double)], C.c_int),
    ("jdem_contacts", [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)], C.c_int),
    ("jdem_neighbor_list", [C.c_void_p, C.c_float, C.c_int32, C.c_void_p, C.POINTER(C.c_int32)], C.c_int),
    ("jdem_domain_state", [C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    ("jdem_stats", [C.c_void_p, C.POINTER(Stats)], C.c_int),
    ("jdem_stream", [C.c_void_p], C.c_void_p),
    ("jdem_set_stream", [C.c_void_p, C.c_void_p], C.c_int),
    ("jdem_shape", [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int32)], C.c_int),
    ("jdem_set_barrier_limit", [C.c_void_p, C.c_uint32, C.c_uint32], C.c_int),
    ("jdem_download_device_async", [C.c_void_p, C.POINTER(HostState)], C.c_int),
    ("jdem_host_register", [C.c_void_p, C.c_size_t], C.c_int),
    ("jdem_host_unregister", [C.c_void_p], C.c_int),
    ("jdem_integrate", [C.c_int32, C.c_int64, C.c_int32, C.c_int32, C.c_int32, C.c_float] + [C.c_void_p] * 10,
     C.c_int),
    ("jdem_domain_apply", [C.c_int32, C.c_int64, C.c_int32, C.c_float, C.c_float] + [C.c_void_p] * 13, C.c_int),
    ("jdem_force_manager_apply", [C.c_int32, C.c_int64] + [C.c_void_p] * 8, C.c_int),
]

EXPORTED = [p[0] for p in _PROTOS]


def load(path: Optional[os.PathLike] = None) -> C.CDLL:
    """Load the engine library (once).  Raises if it is missing."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build the CUDA engine first "
            "(python -c 'import __graft_entry__ as g; g.build()' or python jaxdem_gb300/build.py)"
        )
    lib = C.CDLL(str(p))
    for name, argt, rest in _PROTOS:
        fn = getattr(lib, name)
        fn.argtypes = argt
        fn.restype = rest
    if path is None:
        _LIB = lib
    return lib


def _ptr(a: Optional[np.ndarray]) -> Optional[int]:
    return None if a is None else a.ctypes.data


class Engine:
    """One device handle: several independent systems of the same dimension.

    ``systems`` is a sequence of dicts with keys ``n``, ``domain``,
    ``linear``, ``rotation``, ``dt``, ``box_size``, ``anchor``,
    ``restitution``, ``gravity``, ``cell_size``, ``search_range``.
    """

    def __init__(self, dim: int, systems: Sequence[dict], young_eff: np.ndarray, skin: float = 0.0,
                 bond_width: int = 0, interact_same_bond_id: bool = False, chunk_steps: int = 50,
                 device: int = 0, neighbor_list=True, graph_mode: int = 0, force_law: str = "spring",
                 material_props: Optional[np.ndarray] = None, prune_skin: float = 0.0,
                 brick_particles: int = 0, force_block: int = 0, small_lanes: int = 0):
        """``young_eff`` is the (M, M) pair constant of ``force_law``: the spring's k,
        (4/3) E* for ``"hertz"`` (``forces.hertz_pair_constant``), or the damping ratio
        beta for ``"cundallstrack"``, which also takes ``material_props`` (M, 4)
        (``forces.cundall_strack_tables``)."""
        self.lib = load()
        self.dim = int(dim)
        self.n_per_system = [int(s["n"]) for s in systems]
        self.P = int(sum(self.n_per_system))
        self.S = len(systems)
        descs = (SystemDesc * self.S)()
        for k, s in enumerate(systems):
            d = descs[k]
            d.n = int(s["n"])
            d.domain = DOMAIN[s.get("domain", "periodic")]
            d.linear_integrator = LINEAR[s.get("linear", "verlet")]
            d.rotation_integrator = ROTATION[s.get("rotation", "")]
            d.dt = float(s.get("dt", 0.005))
            box = np.zeros(3, np.float32)
            anc = np.zeros(3, np.float32)
            grav = np.zeros(3, np.float32)
            box[: self.dim] = np.asarray(s.get("box_size", np.ones(self.dim)), np.float32)
            anc[: self.dim] = np.asarray(s.get("anchor", np.zeros(self.dim)), np.float32)
            grav[: self.dim] = np.asarray(s.get("gravity", np.zeros(self.dim)), np.float32)
            for a in range(3):
                d.box_size[a] = float(box[a])
                d.anchor[a] = float(anc[a])
                d.gravity[a] = float(grav[a])
            d.restitution = float(s.get("restitution", 1.0))
            d.cell_size = float(s.get("cell_size", 1.0))
            d.search_range = int(s.get("search_range", 1))
        self._young = np.ascontiguousarray(young_eff, np.float32)
        cfg = Config()
        cfg.dim = self.dim
        cfg.n_systems = self.S
        cfg.systems = descs
        cfg.skin = float(skin)
        cfg.n_materials = int(self._young.shape[0])
        cfg.young_eff = self._young.ctypes.data_as(C.POINTER(C.c_float))
        cfg.bond_width = int(bond_width)
        cfg.interact_same_bond_id = int(bool(interact_same_bond_id))
        cfg.chunk_steps = int(chunk_steps)
        cfg.device = int(device)
        # True: list with automatic capacity; False: cell traversal every step;
        # an int > 0: list with that initial capacity
        cfg.neighbor_list = (-1 if neighbor_list is False else
                             (0 if neighbor_list is True else int(neighbor_list)))
        cfg.graph_mode = int(graph_mode)
        if force_law not in FORCE_LAW:
            raise ValueError(f"force_law must be one of {sorted(FORCE_LAW)}")
        cfg.force_law = FORCE_LAW[force_law]
        # inner-list margin of the dynamic pruning (0: skin / 3, < 0: off)
        cfg.prune_skin = float(prune_skin)
        # particles per shared-memory brick of the list build (0: 240, 60 at most 32768 particles)
        cfg.brick_particles = int(brick_particles)
        # threads per block of the fused force kernel above 32768 slots (0: 128), and
        # lanes per slot of the small-system force kernels (0: 8)
        cfg.force_block = int(force_block)
        cfg.small_lanes = int(small_lanes)
        self.force_law = force_law
        self._props = None
        if material_props is not None:
            self._props = np.ascontiguousarray(material_props, np.float32).reshape(-1, 4)
            if self._props.shape[0] != self._young.shape[0]:
                raise ValueError("material_props must have one row of 4 per material")
            cfg.material_props = self._props.ctypes.data_as(C.POINTER(C.c_float))
        self._descs = descs
        h = C.c_void_p()
        rc = self.lib.jdem_create(C.byref(cfg), C.byref(h))
        if rc != JDEM_OK:
            raise JdemError(rc, "jdem_create failed (see stderr)")
        self.h = h
        self.bond_width = int(bond_width)

    # -- lifetime -------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.jdem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int) -> None:
        if rc != JDEM_OK:
            msg = self.lib.jdem_last_error(self.h)
            raise JdemError(rc, msg.decode() if msg else "")

    # -- state transfer -------------------------------------------------
    def upload(self, pos, rad, mass, vel=None, force=None, q=None, ang_vel=None, torque=None,
               inertia=None, mat_id=None, fixed=None, bond_id=None, pos_p=None, clump_id=None) -> None:
        """Copy one State (concatenated systems) to the device.  Rigid clumps: ``pos_p``
        (body-frame offsets) and ``clump_id`` (clump index within each system); members
        carry their clump's pos_c, vel, q, ang_vel, mass and inertia."""
        P, d = self.P, self.dim
        ad = 3 if d == 3 else 1
        keep = []

        def arr(x, dt, shape):
            if x is None:
                return None
            a = np.ascontiguousarray(np.asarray(x, dt).reshape(shape))
            keep.append(a)
            return a

        hs = HostState()
        hs.pos_c = _ptr(arr(pos, np.float32, (P, d)))
        hs.vel = _ptr(arr(vel, np.float32, (P, d)))
        hs.force = _ptr(arr(force, np.float32, (P, d)))
        hs.q = _ptr(arr(q, np.float32, (P, 4)))
        hs.ang_vel = _ptr(arr(ang_vel, np.float32, (P, ad)))
        hs.torque = _ptr(arr(torque, np.float32, (P, ad)))
        hs.rad = _ptr(arr(rad, np.float32, (P,)))
        hs.mass = _ptr(arr(mass, np.float32, (P,)))
        hs.inertia = _ptr(arr(inertia, np.float32, (P, ad)))
        hs.mat_id = _ptr(arr(mat_id, np.int32, (P,)))
        hs.fixed = _ptr(arr(None if fixed is None else np.asarray(fixed).astype(np.uint8), np.uint8, (P,)))
        if self.bond_width > 0:
            hs.bond_id = _ptr(arr(bond_id, np.int32, (P, self.bond_width)))
        hs.pos_p = _ptr(arr(pos_p, np.float32, (P, d)))
        hs.clump_id = _ptr(arr(clump_id, np.int32, (P,)))
        self._check(self.lib.jdem_upload(self.h, C.byref(hs)))

    def download(self, out: Optional[dict] = None) -> dict:
        """Read pos_c, vel, force, q, ang_vel, torque back (caller order)."""
        P, d = self.P, self.dim
        ad = 3 if d == 3 else 1
        if out is None:
            out = {
                "pos_c": np.empty((P, d), np.float32),
                "vel": np.empty((P, d), np.float32),
                "force": np.empty((P, d), np.float32),
                "q": np.empty((P, 4), np.float32),
                "ang_vel": np.empty((P, ad), np.float32),
                "torque": np.empty((P, ad), np.float32),
            }
        hs = HostState()
        for k in ("pos_c", "vel", "force", "q", "ang_vel", "torque"):
            if k in out and out[k] is not None:
                assert out[k].flags["C_CONTIGUOUS"] and out[k].dtype == np.float32
                setattr(hs, k, out[k].ctypes.data)
        self._check(self.lib.jdem_download(self.h, C.byref(hs)))
        return out

    FRAME_FIELDS = ("pos_c", "vel", "force", "q", "ang_vel", "torque")

    def rollout(self, strides, fields=("pos_c", "vel", "force", "q", "ang_vel", "torque"), out=None,
                ring: int = 0, boxes: bool = True) -> dict:
        """Run ``strides[t]`` steps per frame and save the selected fields after each
        (``jdem_rollout``).  Returns arrays of shape ``(T, P, ...)`` in caller order, plus
        ``box`` / ``anchor`` of shape ``(T, S, dim)`` when ``boxes``.

        ``out`` may hold preallocated destinations: numpy arrays (page-locked ones are
        written by the copy engine directly) or CUDA tensors exposing ``data_ptr()``
        (then every particle field must be a CUDA tensor and frames stay in HBM)."""
        st = np.ascontiguousarray(np.asarray(strides, np.int64).reshape(-1))
        T, P, d = len(st), self.P, self.dim
        ad = 3 if d == 3 else 1
        tails = {"pos_c": (d,), "vel": (d,), "force": (d,), "q": (4,), "ang_vel": (ad,), "torque": (ad,)}
        for k in fields:
            if k not in tails:
                raise ValueError(f"unknown frame field {k!r}")
        out = dict(out or {})
        fr = Frames()
        device = None
        for k in fields:
            a = out.get(k)
            if a is None:
                a = out[k] = np.empty((T, P, *tails[k]), np.float32)
            if hasattr(a, "data_ptr"):
                if tuple(a.shape) != (T, P, *tails[k]) or not a.is_contiguous() or str(a.dtype) != "torch.float32":
                    raise ValueError(f"frame field {k}: expected contiguous float32 {(T, P, *tails[k])}")
                dev, ptr = True, a.data_ptr()
            else:
                if a.shape != (T, P, *tails[k]) or not a.flags["C_CONTIGUOUS"] or a.dtype != np.float32:
                    raise ValueError(f"frame field {k}: expected contiguous float32 {(T, P, *tails[k])}")
                dev, ptr = False, a.ctypes.data
            if device is not None and dev != device:
                raise ValueError("frame fields must be all host arrays or all device tensors")
            device = dev
            setattr(fr, k, ptr if a.size else None)
        fr.device_ptrs = 1 if device else 0
        fr.ring = int(ring)
        if boxes:
            out["box"] = np.zeros((T, self.S, 3), np.float32)
            out["anchor"] = np.zeros((T, self.S, 3), np.float32)
            fr.box, fr.anchor = out["box"].ctypes.data, out["anchor"].ctypes.data
        self._check(self.lib.jdem_rollout(self.h, st.ctypes.data if T else None, T, C.byref(fr)))
        if boxes:
            out["box"], out["anchor"] = out["box"][..., :d], out["anchor"][..., :d]
        return out

    # -- work -------------------------------------------------------------
    def step(self, n: int) -> None:
        self._check(self.lib.jdem_step(self.h, int(n)))

    def step_async(self, n: int) -> None:
        self._check(self.lib.jdem_step_async(self.h, int(n)))

    def sync(self) -> None:
        self._check(self.lib.jdem_sync(self.h))

    def step_timed(self, n: int) -> tuple[float, float]:
        tot, frc = C.c_double(), C.c_double()
        self._check(self.lib.jdem_step_timed(self.h, int(n), C.byref(tot), C.byref(frc)))
        return tot.value, frc.value

    def compute_force(self) -> None:
        self._check(self.lib.jdem_compute_force(self.h))

    def energy(self, per_system: bool = False) -> np.ndarray:
        if per_system:
            out = np.zeros(4 * self.S, np.float64)
            self._check(self.lib.jdem_energy_per_system(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
            return out.reshape(self.S, 4)
        out = np.zeros(4, np.float64)
        self._check(self.lib.jdem_energy(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def contacts(self) -> np.ndarray:
        cnt = C.c_int64()
        self._check(self.lib.jdem_contacts(self.h, None, 0, C.byref(cnt)))
        n = cnt.value
        pairs = np.zeros((max(n, 1), 2), np.int32)
        self._check(self.lib.jdem_contacts(self.h, pairs.ctypes.data, n, C.byref(cnt)))
        return pairs[:n].astype(np.int64)

    def neighbor_list(self, cutoff: float, max_neighbors: int) -> tuple[np.ndarray, bool]:
        out = np.full((self.P, max(int(max_neighbors), 0)), -1, np.int32)
        ovf = C.c_int32()
        ptr = out.ctypes.data if out.size else None
        self._check(self.lib.jdem_neighbor_list(self.h, float(cutoff), int(max_neighbors), ptr, C.byref(ovf)))
        return out.astype(np.int64), bool(ovf.value)

    def domain_state(self) -> tuple[np.ndarray, np.ndarray]:
        box = np.zeros((self.S, 3), np.float32)
        anc = np.zeros((self.S, 3), np.float32)
        self._check(self.lib.jdem_domain_state(self.h, box.ctypes.data, anc.ctypes.data))
        return box[:, : self.dim], anc[:, : self.dim]

    def stats(self) -> dict:
        st = Stats()
        self._check(self.lib.jdem_stats(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in Stats._fields_}

    def stream(self) -> int:
        return int(self.lib.jdem_stream(self.h) or 0)

    def set_barrier_limit(self, spins: int, extra_arrivals: int = 0) -> None:
        """Fault-path control of the many-step grid barrier (tests of the timeout path)."""
        self._check(self.lib.jdem_set_barrier_limit(self.h, int(spins), int(extra_arrivals)))

    def set_stream(self, stream: int) -> None:
        """Queue later work on ``stream`` (a ``cudaStream_t`` as an int, e.g.
        ``torch.cuda.Stream().cuda_stream``); 0 returns to the handle's own stream."""
        self._check(self.lib.jdem_set_stream(self.h, C.c_void_p(int(stream)) if stream else None))

    _DEVICE_FIELDS = ("pos_c", "vel", "force", "q", "ang_vel", "torque", "rad", "mass", "inertia", "mat_id",
                      "fixed", "bond_id", "pos_p", "clump_id")

    def _device_state(self, arrays: dict) -> HostState:
        hs = HostState()
        for k, a in arrays.items():
            if k not in self._DEVICE_FIELDS:
                raise ValueError(f"unknown state field {k!r}")
            if a is None:
                continue
            if not hasattr(a, "data_ptr") or not a.is_cuda or not a.is_contiguous():
                raise ValueError(f"{k}: expected a contiguous CUDA tensor")
            setattr(hs, k, a.data_ptr())
        return hs

    def upload_device(self, **arrays) -> None:
        """``jdem_upload_device`` from contiguous CUDA tensors in the reference layout
        (float32; int32 ``mat_id``/``bond_id``/``clump_id``, uint8 ``fixed``)."""
        self._check(self.lib.jdem_upload_device(self.h, C.byref(self._device_state(arrays))))

    def download_device(self, wait: bool = True, **arrays) -> None:
        """Copy pos_c / vel / force / q / ang_vel / torque into CUDA tensors; with
        ``wait=False`` the copies are only queued on the active stream."""
        fn = self.lib.jdem_download_device if wait else self.lib.jdem_download_device_async
        self._check(fn(self.h, C.byref(self._device_state(arrays))))


def host_register(a: np.ndarray) -> None:
    """Page-lock a numpy array for asynchronous copies."""
    rc = load().jdem_host_register(a.ctypes.data, a.nbytes)
    if rc != JDEM_OK:
        raise JdemError(rc, "cudaHostRegister failed")


def host_unregister(a: np.ndarray) -> None:
    load().jdem_host_unregister(a.ctypes.data)
