"""Dynamic pruning of the Verlet list (systems above 32768 slots).

Between re-sorts the force kernel walks an inner list: the entries of the full list within
r_i + r_j + prune_skin of the positions at its build, rebuilt from the full list whenever
the accumulated drift exceeds prune_skin / 2.  Entries farther than the contact distance
add nothing to a particle's force, and the inner list keeps the full list's order, so the
contact sums see the same nonzero terms in the same order: trajectories with pruning must
equal trajectories without it bit for bit, for any prune skin.
"""

from __future__ import annotations

import numpy as np
import pytest

from jaxdem_gb300 import workloads as W
from jaxdem_gb300._lib import Engine

pytestmark = pytest.mark.gpu

K = np.array([[W.K_SPRING]], np.float32)


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def _run(w, steps, skin, prune_skin, graph_mode=0):
    eng = Engine(w.dim, [w.desc()], K, skin=skin, prune_skin=prune_skin, graph_mode=graph_mode)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.step(steps)
        out = eng.download()
        st = eng.stats()
    finally:
        eng.close()
    return out, st


@pytest.mark.parametrize("case,prune_skin,graph_mode", [
    ("bidisperse3d", 0.0, 0),      # the default prune skin (skin / 3), conditional graphs
    ("bidisperse3d", 0.02, 2),     # a tiny prune skin: a prune nearly every step, direct launches
    ("reflect2d", 0.0, 0),         # reflecting walls and gravity
])
def test_pruned_list_trajectory_equals_full_list(case, prune_skin, graph_mode):
    if case == "bidisperse3d":
        w = W.c2(N=131072, seed=61)
    else:
        w = W.c3(N=65536, seed=62)
        w.vel = np.random.default_rng(7).normal(0, 0.3, size=w.vel.shape).astype(np.float32)
    skin = 0.65 * float(w.rad.max())
    steps = 120
    pruned, st_p = _run(w, steps, skin, prune_skin, graph_mode)
    full, st_f = _run(w, steps, skin, -1.0, graph_mode)
    assert st_f["prunes"] == 0
    assert st_p["prunes"] > 0, st_p
    if prune_skin == 0.0:
        assert st_p["prunes"] < steps, st_p  # most steps walk the inner list
    assert st_p["rebuilds"] == st_f["rebuilds"]
    assert np.array_equal(pruned["pos_c"], full["pos_c"])
    assert np.array_equal(pruned["vel"], full["vel"])
    assert np.array_equal(pruned["force"], full["force"])
