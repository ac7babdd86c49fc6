"""The allocation-free force entry point against the regular one.

``jdem_compute_force_noalloc`` is for callers that cannot allocate device
memory while they run (an XLA FFI handler inside XLA's preallocated pool,
code inside another framework's memory budget).  It keeps its scratch in one
fixed device array of the library.  This test calls it through the C ABI on
two different systems in a row (the second call finds the first call's
leftovers in the shared scratch) and checks each result against
``jdem_compute_force`` within the force tolerance of the other parity tests.
The file name sorts last so that a run stopping at the first failure has
already run every other test.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from jaxdem_gb300 import workloads as W
from jaxdem_gb300._lib import Engine, load
from tests.helpers import force_err

pytestmark = pytest.mark.gpu

F32 = np.float32
MAX_P = 65536


def _fn():
    lib = load()
    fn = lib.jdem_compute_force_noalloc
    fn.argtypes = [C.c_int32, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


DOMAIN = {"free": 0, "periodic": 1, "reflect": 2}


def _noalloc_force(w):
    import torch

    dev = torch.device("cuda:0")
    pos = torch.from_numpy(np.ascontiguousarray(w.pos)).to(dev)
    rad = torch.from_numpy(np.ascontiguousarray(w.rad)).to(dev)
    out = torch.full((w.N, w.dim), float("nan"), dtype=torch.float32, device=dev)
    box = np.ascontiguousarray(w.box_size, F32)
    anc = np.ascontiguousarray(w.anchor, F32)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = _fn()(w.dim, w.N, DOMAIN[w.domain], box.ctypes.data, anc.ctypes.data, float(W.K_SPRING),
               pos.data_ptr(), rad.data_ptr(), out.data_ptr(), stream)
    assert rc == 0, f"jdem_compute_force_noalloc returned {rc}"
    torch.cuda.synchronize(dev)
    return out.cpu().numpy()


def _regular_force(w):
    eng = Engine(w.dim, [w.desc()], np.array([[W.K_SPRING]], F32), skin=0.05)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.compute_force()
        return eng.download()["force"]
    finally:
        eng.close()


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def test_noalloc_matches_regular_entry_point_twice_in_a_row():
    rng = np.random.Generator(np.random.PCG64(21))
    first = W.periodic_system("a", rng, 8192, 3, rng.choice([0.5, 0.7], size=8192), 0.55, 0.1, 1e-3, 1)
    second = W.c3(N=3000, seed=22)  # 2D reflect after 3D periodic: stale scratch from the first call
    for w in (first, second):
        got = _noalloc_force(w)
        ref = _regular_force(w)
        assert np.isfinite(got).all()
        err = force_err(got, ref)
        assert err <= 1e-5, f"{w.name}: noalloc vs jdem_compute_force err {err}"


MAX_CELLS = 131072


def _check(w):
    got = _noalloc_force(w)
    ref = _regular_force(w)
    assert np.isfinite(got).all()
    err = force_err(got, ref)
    assert err <= 1e-5, f"{w.name}: noalloc vs jdem_compute_force err {err}"
    return got


def test_noalloc_free_domain():
    """Free domain: the grid's origin and extent come from the device bounding box."""
    rng = np.random.Generator(np.random.PCG64(23))
    w = W.periodic_system("free", rng, 4000, 3, rng.choice([0.5, 0.7], size=4000), 0.4, 0.1, 1e-3, 1)
    w.domain = "free"
    w.pos = (w.pos - 37.5).astype(F32)  # away from the origin: the bounding box sets the frame
    _check(w)


def test_noalloc_coarsens_a_dilute_grid():
    """A dilute periodic box whose grid at 2 r_max has far more than 131072 cells: the
    device coarsens the grid until it fits the fixed scratch, and the forces still match."""
    rng = np.random.Generator(np.random.PCG64(24))
    N = 30000
    w = W.periodic_system("dilute", rng, N, 3, np.full(N, 0.5), 0.004, 0.1, 1e-3, 1)
    # make some contacts: pairs of overlapping spheres
    w.pos[1::2] = (w.pos[0::2] + rng.uniform(-0.5, 0.5, size=w.pos[0::2].shape)).astype(F32)
    L = float(w.box_size[0])
    uncoarsened = int(np.floor(L / (2 * float(w.rad.max())))) ** 3
    assert uncoarsened > 10 * MAX_CELLS, "the input must need coarsening"
    got = _check(w)
    assert np.abs(got).max() > 1.0, "the case should have contacts"


def test_noalloc_clustered_cells_keep_a_deterministic_order():
    """A free-domain cluster with one far-away sphere: the coarsened grid puts thousands of
    spheres in one cell, which takes the bitmap ordering path.  Two calls give identical
    forces bit for bit, and both match the regular entry point."""
    rng = np.random.Generator(np.random.PCG64(25))
    N = 12000
    w = W.periodic_system("cluster", rng, N, 3, rng.choice([0.5, 0.7], size=N), 0.5, 0.1, 1e-3, 1)
    w.domain = "free"
    w.pos[-1] = np.array([5.0e3, -4.0e3, 3.0e3], F32)
    a = _check(w)
    b = _noalloc_force(w)
    assert np.array_equal(a, b)


def test_noalloc_rejects_oversized_input():
    rc = _fn()(3, MAX_P + 1, 1, None, None, 1.0, None, None, None, None)
    assert rc == 2  # JDEM_ERR_CAPACITY_OVERFLOW, before any device work


def test_noalloc_rejects_negative_n():
    rc = _fn()(3, -5, 1, None, None, 1.0, None, None, None, None)
    assert rc == 1  # JDEM_ERR_BAD_ARG
