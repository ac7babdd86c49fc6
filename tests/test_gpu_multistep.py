"""Small systems run each chunk of steps as one cooperative many-step launch
(jaxdem_gb300/csrc/jdem_multi.cu): one grid barrier per step instead of two
kernel launches, re-sorts between launches in a while node.

Its steps are k_force_small's operations followed by k_fin's bound update,
in the same order, so a trajectory equals the launch-per-step path
(graph_mode 2) bit for bit, re-sort for re-sort.  Checked in 3D periodic and
2D reflect-with-gravity boxes, for the spring and Hertz laws, with two
materials (the general pair path), across chunk boundaries and partial
chunks; systems too large for one resident cooperative grid keep the
per-step graphs.
"""

from __future__ import annotations

import numpy as np
import pytest

from jaxdem_gb300 import workloads as W
from jaxdem_gb300._lib import Engine
from oracle import dem_ref as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def run(w, young, graph_mode, calls, skin, mat=None, law="spring", chunk=50):
    eng = Engine(w.dim, [w.desc()], young, skin=skin, chunk_steps=chunk, graph_mode=graph_mode, force_law=law)
    try:
        kw = {} if mat is None else {"mat_id": mat}
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel, **kw)
        for n in calls:
            eng.step(n)
        out = eng.download()
        st = eng.stats()
    finally:
        eng.close()
    return out, st


def same_trajectory(w, young, skin, calls=(137, 163), **kw):
    a, sa = run(w, young, 0, calls, skin, **kw)
    b, sb = run(w, young, 2, calls, skin, **kw)
    assert sa["many_step"] == 1 and sb["many_step"] == 0
    assert sa["rebuilds"] == sb["rebuilds"] and sa["rebuilds"] > 2
    for k in ("pos_c", "vel", "force"):
        assert np.array_equal(a[k], b[k]), k
    return a, sa


def test_c1_periodic_spring_bit_identical():
    w = W.c1(N=4096, seed=71)
    same_trajectory(w, np.array([[W.K_SPRING]], np.float32), skin=0.02)


def test_reflect_2d_gravity_bit_identical():
    w = W.c3(N=6000, seed=72)
    same_trajectory(w, np.array([[W.K_SPRING]], np.float32), skin=0.05, calls=(120, 1, 79))


def test_hertz_bit_identical():
    w = W.c1(N=3000, seed=73)
    same_trajectory(w, R.hertz_constant([1e3], [0.3]), skin=0.02, law="hertz")


def test_two_materials_bit_identical():
    w = W.c1(N=2500, seed=74)
    young = np.array([[W.K_SPRING, 0.5 * W.K_SPRING], [0.5 * W.K_SPRING, 2 * W.K_SPRING]], np.float32)
    mat = np.random.default_rng(3).integers(0, 2, w.N).astype(np.int32)
    same_trajectory(w, young, skin=0.02, mat=mat)


def test_short_chunks_and_single_steps():
    """Chunks of 7 steps and calls of one step (the final step of a call always takes
    the per-step path) agree with direct launches."""
    w = W.c1(N=2048, seed=75)
    young = np.array([[W.K_SPRING]], np.float32)
    a, sa = run(w, young, 0, (1, 2, 3, 40, 1, 64), 0.02, chunk=7)
    b, sb = run(w, young, 2, (1, 2, 3, 40, 1, 64), 0.02, chunk=7)
    assert sa["many_step"] == 1 and sa["rebuilds"] == sb["rebuilds"]
    for k in ("pos_c", "vel", "force"):
        assert np.array_equal(a[k], b[k]), k


def test_several_systems_bit_identical():
    """Three periodic boxes of different sizes and densities in one handle (the system
    table the many-step kernel keeps in shared memory)."""
    rng = np.random.Generator(np.random.PCG64(77))
    ws = [W.periodic_system(f"s{i}", rng, n, 3, rng.choice([0.5, 0.6], size=n), phi, 0.3, 1e-3, 10)
          for i, (n, phi) in enumerate([(1500, 0.35), (700, 0.5), (2300, 0.42)])]
    cat = lambda k: np.concatenate([getattr(w, k) for w in ws])
    young = np.array([[W.K_SPRING]], np.float32)
    outs, sts = [], []
    for mode in (0, 2):
        eng = Engine(3, [w.desc() for w in ws], young, skin=0.03, graph_mode=mode)
        try:
            eng.upload(pos=cat("pos"), rad=cat("rad"), mass=cat("mass"), vel=cat("vel"))
            eng.step(150)
            eng.step(73)
            outs.append(eng.download())
            sts.append(eng.stats())
        finally:
            eng.close()
    assert sts[0]["many_step"] == 1 and sts[1]["many_step"] == 0
    assert sts[0]["rebuilds"] == sts[1]["rebuilds"] > 2
    for k in ("pos_c", "vel", "force"):
        assert np.array_equal(outs[0][k], outs[1][k]), k


def test_large_system_keeps_per_step_graphs():
    w = W.c1(N=40000, seed=76)
    _, st = run(w, np.array([[W.K_SPRING]], np.float32), 0, (60,), 0.1)
    assert st["many_step"] == 0
