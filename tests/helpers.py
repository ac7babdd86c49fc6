"""Shared helpers for the parity tests: oracle systems and error metrics."""

from __future__ import annotations

import numpy as np

from oracle import dem_ref as R

F32 = np.float32


def force_err(gpu, ref):
    """max_i |F_gpu - F_ref| / max(|F_ref|, 1e-3 rms|F_ref|) with float64 norms."""
    ref = np.asarray(ref, np.float64)
    gpu = np.asarray(gpu, np.float64)
    na = np.linalg.norm(ref, axis=-1)
    rms = np.sqrt(np.mean(na ** 2)) if na.size else 0.0
    floor = max(1e-3 * rms, 1e-30)
    return float((np.linalg.norm(gpu - ref, axis=-1) / np.maximum(na, floor)).max()) if na.size else 0.0


def global_force_err(gpu, ref):
    """||F_gpu - F_ref||_2 / ||F_ref||_2 over all particles, float64 norms (0 without forces).
    The per-particle floored bar of force_err implies the same bar here."""
    ref = np.asarray(ref, np.float64)
    gpu = np.asarray(gpu, np.float64)
    nr = np.linalg.norm(ref)
    return float(np.linalg.norm(gpu - ref) / nr) if nr > 0 else 0.0


def min_image_diff(a, b, box=None):
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    if box is not None:
        box = np.asarray(box, np.float64)
        d = d - box * np.round(d / box)
    return np.abs(d).max() if d.size else 0.0


def osystem(w, domain=None, cell_size=None, search_range=None, young=None, linear="verlet", rotation="",
            gravity=None):
    dim = w.dim
    cell, mask = R.cell_list_create(w.rad, dim, cell_size=cell_size, search_range=search_range)
    return R.OSystem(dim=dim, domain=domain or w.domain, box_size=np.asarray(w.box_size, F32).copy(),
                     anchor=np.asarray(w.anchor, F32).copy(),
                     young_eff=np.array([[1e3]], F32) if young is None else np.asarray(young, F32),
                     dt=F32(w.dt), cell_size=cell, neighbor_mask=mask,
                     gravity=np.asarray(w.gravity if gravity is None else gravity, F32),
                     restitution=F32(w.restitution), linear=linear, rotation=rotation)


def ostate(w, **kw):
    return R.make_state(w.pos, vel=w.vel, rad=w.rad, mass=w.mass, **kw)


# ---------------------------------------------------------------- golden vectors of the reference
# tests/golden/reference_<case>.npz hold inputs and outputs of JaxDEM's own State/System code
# (tests/golden/make_reference_golden.py); these helpers turn a case into oracle objects.

def load_reference_case(name, x64=False):
    import json
    from pathlib import Path

    p = Path(__file__).resolve().parent / "golden" / f"reference_{name}{'_x64' if x64 else ''}.npz"
    z = np.load(p)
    d = {k: z[k] for k in z.files}
    d["meta"] = json.loads(str(d["meta"]))
    return d


def reference_case_names():
    from pathlib import Path

    g = Path(__file__).resolve().parent / "golden"
    return sorted(p.stem[len("reference_"):] for p in g.glob("reference_*.npz") if not p.stem.endswith("_x64"))


def reference_osystem(d, dtype=np.float32):
    """The oracle's System for a golden case (the reference's cell list, laws and integrators)."""
    m = d["meta"]
    dim = m["dim"]
    _, mask = R.cell_list_create(d["rad"], dim)
    law = m.get("law", "spring")
    young = np.asarray(d["young_eff"], dtype)
    if law == "hertz":
        young = R.hertz_constant(np.asarray(m.get("young", [1.0e3])), np.full(len(m.get("young", [1.0e3])), 0.3))
    props = None
    if law == "cundallstrack":
        young, props = reference_cs_tables(d)
    grav = np.zeros(dim, dtype) if not m.get("gravity") else np.asarray(m["gravity"], dtype)
    return R.OSystem(dim=dim, domain=m["domain"], box_size=np.asarray(d["box"], dtype).copy(),
                     anchor=np.asarray(d["anchor"], dtype).copy(), young_eff=np.asarray(young, dtype),
                     dt=dtype(m["dt"]), cell_size=dtype(d["cell_size"]), neighbor_mask=mask, gravity=grav,
                     restitution=dtype(m.get("restitution", 1.0)), linear=m.get("linear", "verlet"),
                     rotation=m.get("rotation", "verletspiral"), force_law=law,
                     mat_props=None if props is None else np.asarray(props, dtype),
                     nlist=None if m.get("collider", "CellList") != "NeighborList" else R.neighbor_list_collider(
                         d["nl_list_cutoff"], d["nl_list_skin"], int(d["nl_max"]), dtype))


def reference_cs_tables(d):
    """The Cundall-Strack tables of a golden case: the damping ratio beta (M, M) and the
    per-material (young, shear modulus, mu, mu_r) rows, from the case's material lists."""
    m = d["meta"]
    return R.cs_tables(young=m["young"], poisson=m["poisson"], e=m["e"], mu=m["mu"], mu_r=m["mu_r"])


def reference_ostate(d, dtype=np.float32):
    clump = {k: d[k] for k in ("pos_p", "q", "clump_id") if k in d}
    return R.make_state(d["pos"], vel=d["vel"], rad=d["rad"], mass=d["mass"], mat_id=d["mat_id"],
                        ang_vel=d["ang_vel"], inertia=d["inertia"], dtype=dtype, **clump)
