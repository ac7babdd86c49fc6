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
OUT64 = HERE / "_build" / "libjdem_oracle_f64.so"
CFLAGS = ["-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c11"]

DOMAIN = {"free": 0, "periodic": 1, "reflect": 2}
LINEAR = {"": 0, "verlet": 1, "euler": 2}
LAW = {"spring": 0, "hertz": 1}

def build_c(force: bool = False) -> Path:
    """Compile the C restatement twice (float32 and float64; gcc, OpenMP, no FMA contraction)."""
    for out, extra in ((OUT, []), (OUT64, ["-DJDEM_ORACLE_F64"])):
        if not force and out.exists() and out.stat().st_mtime >= SRC.stat().st_mtime:
            continue
        out.parent.mkdir(exist_ok=True)
        tmp = out.with_suffix(".so.tmp")
        cmd = [os.environ.get("CC", "gcc"), *CFLAGS, *extra, str(SRC), "-o", str(tmp), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
        os.replace(tmp, out)
    return OUT


_LIBS = {}


def load_c(f64: bool = False) -> C.CDLL:
    if f64 not in _LIBS:
        build_c()
        lib = C.CDLL(str(OUT64 if f64 else OUT))
        sfx = "_f64" if f64 else ""
        fp = C.POINTER(C.c_double if f64 else C.c_float)
        real = C.c_double if f64 else C.c_float
        step = getattr(lib, "oracle_step" + sfx)
        step.argtypes = [C.c_int, C.c_int64, C.c_int, fp, fp, real, fp, real, real, C.c_int, C.c_int, fp, C.c_int,
                         fp, fp, fp, fp, fp, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, fp, fp, C.c_int]
        step.restype = C.c_int
        force = getattr(lib, "oracle_force" + sfx)
        force.argtypes = [C.c_int, C.c_int64, C.c_int, fp, fp, real, C.c_int, C.c_int, fp, fp, fp, C.c_void_p, fp,
                          C.c_int, C.c_int, C.c_int]
        force.restype = C.c_int
        getattr(lib, "oracle_max_threads" + sfx).restype = C.c_int
        contacts = getattr(lib, "oracle_contacts" + sfx)
        contacts.argtypes = [C.c_int, C.c_int64, C.c_int, fp, fp, real, fp, fp, C.c_void_p, C.c_int64, C.c_int]
        contacts.restype = C.c_int64
        lib.step, lib.force, lib.max_threads = step, force, getattr(lib, "oracle_max_threads" + sfx)
        lib.contacts = contacts
        _LIBS[f64] = lib
    return _LIBS[f64]


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double if a.dtype == np.float64 else C.c_float))


def c_step(dim, pos, vel, force, rad, mass, *, domain, box, anchor, dt, steps, cell_size, search_range=1,
           young=None, gravity=None, restitution=1.0, linear="verlet", mat_id=None, fixed=None, threads=0,
           acc64=False, law="spring"):
    """Run ``steps`` reference steps in place; float32 arrays use the float
    build, float64 arrays the double build.  ``young`` is the force law's pair
    constant (spring k, or (4/3) E* for ``law="hertz"``).  Returns (box, anchor)."""
    f64 = pos.dtype == np.float64
    T = np.float64 if f64 else np.float32
    lib = load_c(f64)
    N = pos.shape[0]
    for a in (pos, vel, force):
        assert a.dtype == T and a.flags["C_CONTIGUOUS"]
    rad = np.ascontiguousarray(rad, T)
    mass = np.ascontiguousarray(mass, T)
    young = np.ascontiguousarray(np.array([[1e3]]) if young is None else young, T)
    box3, anc3, g3 = np.zeros(3, T), np.zeros(3, T), np.zeros(3, T)
    box3[:dim] = box
    anc3[:dim] = anchor
    if gravity is not None:
        g3[:dim] = gravity
    mat = np.zeros(N, np.int32) if mat_id is None else np.ascontiguousarray(mat_id, np.int32)
    fx = np.zeros(N, np.uint8) if fixed is None else np.ascontiguousarray(fixed, np.uint8)
    bo, ao = np.zeros(3, T), np.zeros(3, T)
    rc = lib.step(dim, N, DOMAIN[domain], _p(box3), _p(anc3), float(restitution), _p(g3), float(dt),
                  float(cell_size), int(search_range), young.shape[0], _p(young), LINEAR[linear],
                  _p(pos), _p(vel), _p(force), _p(rad), _p(mass), mat.ctypes.data, fx.ctypes.data,
                  int(steps), int(threads), int(acc64), _p(bo), _p(ao), LAW[law])
    if rc != 0:
        raise RuntimeError(f"oracle_step failed ({rc})")
    return bo[:dim].copy(), ao[:dim].copy()


def c_force(dim, pos, rad, *, domain, box, anchor, cell_size, search_range=1, young=None, mat_id=None,
            threads=0, acc64=False, law="spring"):
    f64 = np.asarray(pos).dtype == np.float64
    T = np.float64 if f64 else np.float32
    lib = load_c(f64)
    pos = np.ascontiguousarray(pos, T)
    N = pos.shape[0]
    rad = np.ascontiguousarray(rad, T)
    young = np.ascontiguousarray(np.array([[1e3]]) if young is None else young, T)
    box3, anc3 = np.zeros(3, T), np.zeros(3, T)
    box3[:dim] = box
    anc3[:dim] = anchor
    mat = np.zeros(N, np.int32) if mat_id is None else np.ascontiguousarray(mat_id, np.int32)
    out = np.zeros((N, dim), T)
    rc = lib.force(dim, N, DOMAIN[domain], _p(box3), _p(anc3), float(cell_size), int(search_range),
                   young.shape[0], _p(young), _p(pos), _p(rad), mat.ctypes.data, _p(out), int(threads), int(acc64),
                   LAW[law])
    if rc != 0:
        raise RuntimeError(f"oracle_force failed ({rc})")
    return out


def c_contacts(dim, pos, rad, *, domain, box, anchor, cell_size, threads=0):
    """Canonical contact set of the C restatement: ``(i < j)`` pairs with
    ``d_sq < (r_i + r_j)^2`` (float32 arithmetic of ``periodic.py:74-79``), as an
    ``(n_pairs, 2)`` int64 array sorted lexicographically."""
    lib = load_c(False)
    pos = np.ascontiguousarray(pos, np.float32)
    rad = np.ascontiguousarray(rad, np.float32)
    N = pos.shape[0]
    box3, anc3 = np.zeros(3, np.float32), np.zeros(3, np.float32)
    box3[:dim] = box
    anc3[:dim] = anchor
    args = (dim, N, DOMAIN[domain], _p(box3), _p(anc3), float(cell_size), _p(pos), _p(rad))
    n = lib.contacts(*args, None, 0, int(threads))
    if n < 0:
        raise RuntimeError("oracle_contacts: allocation failed")
    pairs = np.zeros((max(n, 1), 2), np.int64)
    n2 = lib.contacts(*args, pairs.ctypes.data, n, int(threads))
    if n2 != n:
        raise RuntimeError(f"oracle_contacts: count changed between passes ({n} vs {n2})")
    pairs = pairs[:n]
    order = np.lexsort((pairs[:, 1], pairs[:, 0]))
    return pairs[order]


def max_threads() -> int:
    return int(load_c().max_threads())
