"""Oracle package: CPU restatements of JaxDEM's hot path (TEST INFRASTRUCTURE).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package.  ``dem_ref`` is the numpy restatement;
``jdem_oracle.c`` the C/OpenMP one, built by :func:`build_c` into
``oracle/_build/``.  The reference is pure Python/JAX, so there is no
reference source to compile into ``oracle/_ref``.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "jdem_oracle.c"
OUT = HERE / "_build" / "libjdem_oracle.so"
CFLAGS = ["-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c11"]

DOMAIN = {"free": 0, "periodic": 1, "reflect": 2}
LINEAR = {"": 0, "verlet": 1, "euler": 2}

_LIB = None


def build_c(force: bool = False) -> Path:
    """Compile the C restatement (gcc, OpenMP, no FMA contraction)."""
    if not force and OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [os.environ.get("CC", "gcc"), *CFLAGS, str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


def load_c() -> C.CDLL:
    global _LIB
    if _LIB is None:
        build_c()
        lib = C.CDLL(str(OUT))
        fp = C.POINTER(C.c_float)
        lib.oracle_step.argtypes = [C.c_int, C.c_int64, C.c_int, fp, fp, C.c_float, fp, C.c_float, C.c_float,
                                    C.c_int, C.c_int, fp, C.c_int, fp, fp, fp, fp, fp, C.c_void_p, C.c_void_p,
                                    C.c_int64, C.c_int, C.c_int, fp, fp]
        lib.oracle_step.restype = C.c_int
        lib.oracle_force.argtypes = [C.c_int, C.c_int64, C.c_int, fp, fp, C.c_float, C.c_int, C.c_int, fp, fp, fp,
                                     C.c_void_p, fp, C.c_int, C.c_int]
        lib.oracle_force.restype = C.c_int
        lib.oracle_max_threads.restype = C.c_int
        _LIB = lib
    return _LIB


def _f(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def c_step(dim, pos, vel, force, rad, mass, *, domain, box, anchor, dt, steps, cell_size, search_range=1,
           young=np.array([[1e3]], np.float32), gravity=None, restitution=1.0, linear="verlet", mat_id=None,
           fixed=None, threads=0, acc64=False):
    """Run ``steps`` reference steps in place on float32 arrays; returns (box, anchor)."""
    lib = load_c()
    N = pos.shape[0]
    for a in (pos, vel, force):
        assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    rad = np.ascontiguousarray(rad, np.float32)
    mass = np.ascontiguousarray(mass, np.float32)
    young = np.ascontiguousarray(young, np.float32)
    box3 = np.zeros(3, np.float32)
    anc3 = np.zeros(3, np.float32)
    box3[:dim] = box
    anc3[:dim] = anchor
    g3 = np.zeros(3, np.float32)
    if gravity is not None:
        g3[:dim] = gravity
    mat = np.zeros(N, np.int32) if mat_id is None else np.ascontiguousarray(mat_id, np.int32)
    fx = np.zeros(N, np.uint8) if fixed is None else np.ascontiguousarray(fixed, np.uint8)
    bo = np.zeros(3, np.float32)
    ao = np.zeros(3, np.float32)
    rc = lib.oracle_step(dim, N, DOMAIN[domain], _f(box3), _f(anc3), float(restitution), _f(g3), float(dt),
                         float(cell_size), int(search_range), young.shape[0], _f(young), LINEAR[linear],
                         _f(pos), _f(vel), _f(force), _f(rad), _f(mass), mat.ctypes.data, fx.ctypes.data,
                         int(steps), int(threads), int(acc64), _f(bo), _f(ao))
    if rc != 0:
        raise RuntimeError(f"oracle_step failed ({rc})")
    return bo[:dim].copy(), ao[:dim].copy()


def c_force(dim, pos, rad, *, domain, box, anchor, cell_size, search_range=1,
            young=np.array([[1e3]], np.float32), mat_id=None, threads=0, acc64=False):
    lib = load_c()
    pos = np.ascontiguousarray(pos, np.float32)
    N = pos.shape[0]
    rad = np.ascontiguousarray(rad, np.float32)
    young = np.ascontiguousarray(young, np.float32)
    box3 = np.zeros(3, np.float32)
    anc3 = np.zeros(3, np.float32)
    box3[:dim] = box
    anc3[:dim] = anchor
    mat = np.zeros(N, np.int32) if mat_id is None else np.ascontiguousarray(mat_id, np.int32)
    out = np.zeros((N, dim), np.float32)
    rc = lib.oracle_force(dim, N, DOMAIN[domain], _f(box3), _f(anc3), float(cell_size), int(search_range),
                          young.shape[0], _f(young), _f(pos), _f(rad), mat.ctypes.data, _f(out), int(threads),
                          int(acc64))
    if rc != 0:
        raise RuntimeError(f"oracle_force failed ({rc})")
    return out


def max_threads() -> int:
    return int(load_c().oracle_max_threads())
