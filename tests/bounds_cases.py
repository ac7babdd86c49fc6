"""Child process of ``test_gpu_bounds.py``: the engine's main paths at small sizes.

Loads whichever engine library ``JDEM_LIBRARY`` names (the regular or the bounds-checked
build) and prints one JSON line per case: the sticky device status after the case, the
number of contacts, and a digest of the final positions, velocities and forces.  Cases:
the many-step kernel (4096 spheres), the fused list kernel with the brick list build and
pruning (40,000 spheres, both block shapes, 2D and 3D), two materials with the Hertz law
(the general contact path, pruned), Cundall-Strack with spin and two materials, a
reflecting 2D box with gravity, a free domain (the per-slot list build), 3,000 spheres at
16 lanes a slot, rigid clumps under the spring and Cundall-Strack laws, a batch of twelve
uneven systems, the neighbour-list API and a streamed rollout.
"""

from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

from jaxdem_gb300 import workloads as W  # noqa: E402
from jaxdem_gb300._lib import Engine  # noqa: E402
from jaxdem_gb300.forces import cundall_strack_tables, hertz_pair_constant  # noqa: E402

K = np.array([[W.K_SPRING]], np.float32)


def digest(out: dict) -> str:
    h = hashlib.sha1()
    for k in ("pos_c", "vel", "force"):
        h.update(np.ascontiguousarray(out[k]).tobytes())
    return h.hexdigest()[:16]


def report(tag: str, eng: Engine, extra: dict | None = None) -> None:
    out = eng.download()
    rec = {"case": tag, "status": int(eng.stats()["device_status"]), "contacts": int(len(eng.contacts())),
           "digest": digest(out)}
    rec.update(extra or {})
    print(json.dumps(rec), flush=True)


def run(tag, w, steps=30, young=K, mat_id=None, ang_vel=None, rotation="", **kw):
    d = w.desc()
    d["rotation"] = rotation
    eng = Engine(w.dim, [d], young, **kw)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel, mat_id=mat_id, ang_vel=ang_vel)
        eng.compute_force()
        eng.step(steps)
        report(tag, eng, {"rebuilds": int(eng.stats()["rebuilds"])})
    finally:
        eng.close()


def clumps(n_clumps=1500, seed=61, phi=0.35):
    """Rigid dumbbells and triangles (and single spheres) at random centres, orientations
    and spins in a periodic 3D box, per-member arrays in the reference layout."""
    rng = np.random.default_rng(seed)
    sizes = rng.choice([1, 2, 3], n_clumps, p=[0.2, 0.5, 0.3])
    n = int(sizes.sum())
    rad = rng.uniform(0.4, 0.5, n).astype(np.float32)
    vol = 4.0 / 3.0 * np.pi * rad.astype(np.float64) ** 3
    box = float((vol.sum() / phi) ** (1.0 / 3.0))
    cid = np.repeat(np.arange(n_clumps), sizes)
    offsets = {1: [[0.0, 0.0, 0.0]], 2: [[-0.35, 0.0, 0.0], [0.35, 0.0, 0.0]],
               3: [[-0.3, -0.2, 0.0], [0.3, -0.2, 0.0], [0.0, 0.35, 0.0]]}
    pos_p = np.concatenate([offsets[int(k)] for k in sizes]).astype(np.float32)
    q = rng.normal(size=(n_clumps, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    mass = np.bincount(cid, weights=vol)
    inertia = np.stack([mass * 0.2 + 0.05 * a for a in range(3)], 1)
    arrays = dict(pos=rng.uniform(0, box, (n_clumps, 3))[cid], q=q[cid], vel=rng.normal(0, 0.3, (n_clumps, 3))[cid],
                  ang_vel=rng.normal(0, 1.0, (n_clumps, 3))[cid], mass=mass[cid], inertia=inertia[cid])
    arrays = {k: v.astype(np.float32) for k, v in arrays.items()}
    desc = dict(n=n, domain="periodic", linear="verlet", rotation="verletspiral", dt=1e-3,
                box_size=np.full(3, box, np.float32), anchor=np.zeros(3, np.float32), restitution=1.0,
                gravity=np.zeros(3, np.float32), cell_size=1.0, search_range=1)
    return desc, dict(rad=rad, pos_p=pos_p, clump_id=cid.astype(np.int32), **arrays)


def run_clumps(tag, young, **kw):
    desc, c = clumps()
    eng = Engine(3, [desc], young, skin=0.1, **kw)
    try:
        eng.upload(pos=c["pos"], rad=c["rad"], mass=c["mass"], vel=c["vel"], q=c["q"], ang_vel=c["ang_vel"],
                   inertia=c["inertia"], pos_p=c["pos_p"], clump_id=c["clump_id"],
                   mat_id=(c["clump_id"] % 2).astype(np.int32) if kw.get("force_law") else None)
        eng.compute_force()
        eng.step(30)
        report(tag, eng)
    finally:
        eng.close()


def main() -> None:
    run("many_step_4096", W.c1())
    run("list_pruned_40000", W.c2(N=40000), skin=0.63, prune_skin=0.315)
    run("list_block64_40000", W.c2(N=40000), skin=0.3, prune_skin=-1.0, force_block=64)
    w = W.c2(N=40000)
    mats = np.random.default_rng(3).integers(0, 2, size=40000).astype(np.int32)
    run("hertz_two_materials_40000", w, young=hertz_pair_constant([1e3, 2e3], [0.3, 0.25]), mat_id=mats,
        skin=0.4, force_law="hertz")
    beta, props = cundall_strack_tables([1e3, 3e3], [0.25, 0.3], [0.6, 0.8], [0.4, 0.3], [0.05, 0.1])
    w = W.c2(N=40000)
    spin = np.random.default_rng(4).normal(0.0, 2.0, size=(40000, 3)).astype(np.float32)
    run("cundall_strack_40000", w, young=beta, mat_id=mats, ang_vel=spin, rotation="verletspiral", skin=0.3,
        force_law="cundallstrack", material_props=props)
    w2 = W.periodic_system("p2", np.random.Generator(np.random.PCG64(5)), 40000, 2,
                           np.where(np.arange(40000) % 2 == 0, 0.5, 0.7), 0.7, 0.05, 5e-4, 30)
    run("list_2d_40000", w2, skin=0.5, force_block=256)
    run("reflect_2d_40000", W.c3(N=40000), skin=0.2)
    w = W.c2(N=40000)
    w.domain = "free"
    run("free_40000", w, skin=0.3)
    run("small_lanes16_3000", W.c2(N=3000), skin=0.3, small_lanes=16)
    run_clumps("clumps_spring", K)
    run_clumps("clumps_cundall_strack", beta, force_law="cundallstrack", material_props=props)
    ws = W.c4(n_systems=12, n_max=3000)
    eng = Engine(3, [x.desc() for x in ws], K, skin=0.2)
    try:
        cat = lambda k: np.concatenate([getattr(x, k) for x in ws])  # noqa: E731
        eng.upload(pos=cat("pos"), rad=cat("rad"), mass=cat("mass"), vel=cat("vel"))
        eng.step(30)
        report("batch_12_systems", eng)
    finally:
        eng.close()
    w = W.c1()
    eng = Engine(3, [w.desc()], K)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        nl, overflow = eng.neighbor_list(1.2, 32)
        frames = eng.rollout([1, 2, 3, 4])
        h = hashlib.sha1(np.ascontiguousarray(nl).tobytes() + np.ascontiguousarray(frames["pos_c"]).tobytes())
        report("neighbor_list_rollout_4096", eng, {"nlist": h.hexdigest()[:16], "overflow": bool(overflow)})
    finally:
        eng.close()


if __name__ == "__main__":
    main()
