"""Seeded random configurations against the oracle, through the C ABI.

Each case draws a dimension, domain, size (including both sides of the 32,768-slot switch
between the small-system and the fused list kernel), radius distribution, packing
fraction, skin, prune skin, an initial list capacity that is not a multiple of four (rows
are rounded up), the force law, and the force kernel's block shape or lanes per slot.
The engine must meet the parity bars on each: step-0 forces within 1e-5 (floored
relative, float64-accumulated oracle), the contact set bit for bit, and positions within
1e-4 after eight steps.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from jaxdem_gb300 import workloads as W
from jaxdem_gb300._lib import Engine
from oracle import dem_ref as R
from tests.helpers import force_err, min_image_diff

pytestmark = pytest.mark.gpu

F32 = np.float32
K_SPRING = np.array([[1e3]], F32)
K43 = R.hertz_constant([1e3], [0.3])


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def draw(seed):
    rng = np.random.default_rng(seed)
    dim = int(rng.choice([2, 3]))
    domain = str(rng.choice(["periodic", "periodic", "reflect", "free"]))
    N = int(rng.choice([300, 1500, 32767, 32769, 40000]))
    kind = rng.integers(3)
    if kind == 0:
        rad = np.full(N, 0.5)
    elif kind == 1:
        rad = rng.choice([0.5, 0.7], N)
    else:
        rad = rng.uniform(0.3, 0.6, N)
    phi = float(rng.uniform(0.3, 0.6 if dim == 3 else 0.75))
    w = W.periodic_system("fuzz", np.random.Generator(np.random.PCG64(seed)), N, dim, rad, phi,
                          float(rng.uniform(0.05, 0.5)), 5e-4, 8)
    if domain == "reflect":
        L = w.box_size[0]
        w.pos = np.clip(w.pos, w.rad[:, None] + 1e-3, L - w.rad[:, None] - 1e-3).astype(F32)
        w.gravity = np.zeros(dim, F32)
        w.gravity[1] = -1.0
    w.domain = domain
    params = dict(skin=float(rng.uniform(0.02, 1.2)) * float(rad.max()),
                  prune_skin=float(rng.choice([0.0, -1.0, 0.05])),
                  neighbor_list=int(rng.choice([0, 5, 13, 22])) or True,
                  law=str(rng.choice(["spring", "hertz"])),
                  force_block=int(rng.choice([64, 128, 256])), small_lanes=int(rng.choice([4, 8, 16])))
    return w, params


def _okw(w):
    return dict(domain=w.domain, box=w.box_size, anchor=w.anchor, cell_size=2 * float(w.rad.max()))


@pytest.mark.parametrize("seed", range(24))
def test_random_configuration_meets_the_parity_bars(seed):
    w, p = draw(9000 + seed)
    young = K43 if p["law"] == "hertz" else K_SPRING
    eng = Engine(w.dim, [w.desc()], young, skin=p["skin"], prune_skin=p["prune_skin"],
                 neighbor_list=p["neighbor_list"], force_law=p["law"], force_block=p["force_block"],
                 small_lanes=p["small_lanes"])
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.compute_force()
        f0 = eng.download()["force"]
        pairs = eng.contacts()
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.step(8)
        out = eng.download()
    finally:
        eng.close()
    ref_f = oracle.c_force(w.dim, w.pos, w.rad, young=young, acc64=True, law=p["law"], **_okw(w))
    assert force_err(f0, ref_f) <= 1e-5, p
    ref_pairs = oracle.c_contacts(w.dim, w.pos, w.rad, **_okw(w))
    assert np.array_equal(pairs, ref_pairs), p
    pos, vel, frc = w.pos.copy(), w.vel.copy(), np.zeros_like(w.pos)
    oracle.c_step(w.dim, pos, vel, frc, w.rad, w.mass, dt=w.dt, steps=8, gravity=w.gravity, young=young,
                  restitution=w.restitution, acc64=True, law=p["law"], **_okw(w))
    box = w.box_size if w.domain == "periodic" else None
    assert min_image_diff(out["pos_c"], pos, box) <= 1e-4, p
