"""Golden vectors from JaxDEM's own code, for pinning the oracle and the engine.

JAX cannot be installed here, so this script runs the reference's source tree on the numpy
stand-in for the JAX API in ``tests/golden/jaxshim`` (see its README.txt): the reference's
State.create, System.create, System.step (``jaxdem/system.py:60-82, 701-748``), the cell-list
collider (``jaxdem/colliders/cell_list.py``), the spring / Hertz laws, the Verlet, Euler,
VV-spiral and spiral integrators, the Cundall-Strack law with "elasticfrict" materials, rigid
clumps (per-clump force / torque sums and the reflect domain's clump collisions), the periodic /
reflect / free domains, the thermal energies and ``create_neighbor_list`` execute as written,
with jax.numpy evaluated by numpy.

Every input is drawn here with numpy's PCG64 and stored beside the outputs, so the fixtures
are self-contained:

    python tests/golden/make_reference_golden.py [--reference /path/to/JaxDEM] [--only NAME]

writes ``tests/golden/reference_<case>.npz`` (float32 runs) and ``reference_<case>_x64.npz``
(the same case with ``jax_enable_x64``, for the cases listed in X64_CASES).  Only the
fixture files are read by the tests; this script needs the reference source tree.
"""

from __future__ import annotations

import argparse
import json
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

# name: PCG64 seed, dim, N (spheres, or clumps for radii "clump"), domain, radii ("bi" 0.5/0.7,
# "poly" U[0.4, 0.6], "mono" 0.5, "clump" U[0.4, 0.5]), packing fraction, velocity and spin sigmas,
# dt, gravity, restitution, linear / rotation integrator, force law, the materials' young moduli
# (and poisson / e / mu / mu_r for Cundall-Strack), strides between recorded snapshots,
# neighbour-list cutoff factor
CASES = {
    "per3d_bi": dict(seed=1005, dim=3, N=96, domain="periodic", radii="bi", phi=0.5, vsig=0.1, dt=5e-4, strides=[1, 9, 20],
                     nl=3.0),
    "per2d_poly": dict(seed=1004, dim=2, N=96, domain="periodic", radii="poly", phi=0.7, vsig=0.1, dt=5e-4,
                       strides=[1, 9, 20], nl=2.5),
    "refl2d_grav": dict(seed=1006, dim=2, N=80, domain="reflect", radii="poly", phi=0.5, vsig=0.5, dt=1e-3,
                        gravity=[0.0, -1.0], strides=[1, 9, 30]),
    "refl3d_e08": dict(seed=1007, dim=3, N=64, domain="reflect", radii="bi", phi=0.35, vsig=0.8, dt=1e-3,
                       gravity=[0.0, 0.0, -2.0], restitution=0.8, strides=[1, 9, 30]),
    "free3d": dict(seed=1001, dim=3, N=64, domain="free", radii="bi", phi=0.45, vsig=0.2, dt=5e-4, strides=[1, 9, 20]),
    "rot3d_vvspiral": dict(seed=1009, dim=3, N=64, domain="periodic", radii="mono", phi=0.45, vsig=0.1, dt=1e-3,
                           wsig=2.0, rotation="verletspiral", strides=[1, 9, 10]),
    "rot2d_spiral": dict(seed=1008, dim=2, N=64, domain="periodic", radii="mono", phi=0.6, vsig=0.1, dt=1e-3,
                         wsig=2.0, rotation="spiral", strides=[1, 9, 10]),
    "hertz3d": dict(seed=1002, dim=3, N=64, domain="periodic", radii="bi", phi=0.5, vsig=0.1, dt=5e-4, law="hertz",
                    strides=[1, 9, 10]),
    "mat2_3d": dict(seed=1003, dim=3, N=64, domain="periodic", radii="bi", phi=0.5, vsig=0.1, dt=5e-4,
                    young=[1.0e3, 3.0e3], strides=[1, 9, 10]),
    "euler2d": dict(seed=1000, dim=2, N=64, domain="periodic", radii="poly", phi=0.6, vsig=0.1, dt=5e-4, linear="euler",
                    strides=[1, 9, 10]),
    "tiny3d": dict(seed=1010, dim=3, N=12, domain="periodic", radii="mono", box=2.6, vsig=0.2, dt=1e-3, strides=[1, 9, 20]),
    # Cundall-Strack with two "elasticfrict" materials, random spins (rolling friction active)
    "cs3d": dict(seed=1011, dim=3, N=64, domain="periodic", radii="bi", phi=0.5, vsig=0.3, dt=5e-4, wsig=2.0,
                 law="cundallstrack", strides=[1, 9, 10], young=[1.0e3, 3.0e3], poisson=[0.25, 0.3], e=[0.6, 0.8],
                 mu=[0.4, 0.3], mu_r=[0.05, 0.1]),
    "cs2d_refl": dict(seed=1012, dim=2, N=64, domain="reflect", radii="poly", phi=0.55, vsig=0.5, dt=5e-4, wsig=2.0,
                      gravity=[0.0, -1.0], law="cundallstrack", rotation="spiral", strides=[1, 9, 20],
                      young=[1.0e3, 2.0e3], poisson=[0.3, 0.2], e=[0.5, 0.9], mu=[0.5, 0.2], mu_r=[0.0, 0.2]),
    # rigid clumps of one to three spheres (State.create with pos_p, q, clump_id, mass, inertia)
    "clump3d": dict(seed=1013, dim=3, N=40, domain="periodic", radii="clump", phi=0.35, vsig=0.3, dt=1e-3, wsig=1.0,
                    strides=[1, 9, 20], nl=3.0),
    "clump2d_refl": dict(seed=1014, dim=2, N=40, domain="reflect", radii="clump", phi=0.3, vsig=0.5, dt=1e-3,
                         wsig=1.0, gravity=[0.0, -2.0], strides=[1, 9, 30], nl=2.5),
    # rigid clumps with Cundall-Strack contacts (sphere-centred contact arms, clump velocities)
    "clump_cs3d": dict(seed=1015, dim=3, N=40, domain="periodic", radii="clump", phi=0.35, vsig=0.3, dt=5e-4,
                       wsig=1.0, law="cundallstrack", strides=[1, 9, 20], young=[1.0e3, 3.0e3], poisson=[0.25, 0.3],
                       e=[0.6, 0.8], mu=[0.4, 0.3], mu_r=[0.05, 0.1]),
    # the NeighborList collider (cached Verlet list with skin, rebuilt on displacement)
    "nlist3d": dict(seed=1017, dim=3, N=96, domain="periodic", radii="bi", phi=0.5, vsig=0.3, dt=5e-4,
                    collider="NeighborList", nl_skin=0.15, strides=[1, 9, 30]),
    "nlist2d_refl": dict(seed=1018, dim=2, N=96, domain="reflect", radii="poly", phi=0.6, vsig=0.5, dt=5e-4,
                         gravity=[0.0, -1.0], collider="NeighborList", nl_skin=0.1, strides=[1, 9, 30]),
    "clump_cs2d_refl": dict(seed=1016, dim=2, N=40, domain="reflect", radii="clump", phi=0.3, vsig=0.5, dt=5e-4,
                            wsig=1.0, gravity=[0.0, -2.0], law="cundallstrack", strides=[1, 9, 30],
                            young=[1.0e3, 2.0e3], poisson=[0.3, 0.2], e=[0.5, 0.9], mu=[0.5, 0.2], mu_r=[0.0, 0.2]),
}
X64_CASES = ["per3d_bi", "refl2d_grav"]


def _clumps(rng, n_clumps, dim):
    """Clumps of one to three spheres (radius U[0.4, 0.5]): per-member body-frame offsets,
    the clump index of each member, and per-clump random orientations (w, x, y, z)."""
    sizes = rng.choice([1, 2, 3], n_clumps, p=[0.2, 0.5, 0.3])
    offs = {1: [[0.0, 0.0, 0.0]], 2: [[-0.35, 0.0, 0.0], [0.35, 0.0, 0.0]],
            3: [[-0.3, -0.2, 0.0], [0.3, -0.2, 0.0], [0.0, 0.35, 0.0]]}
    pos_p = np.concatenate([np.asarray(offs[s])[:, :dim] for s in sizes])
    cid = np.repeat(np.arange(n_clumps), sizes)
    if dim == 2:
        a = rng.uniform(0, 2 * np.pi, n_clumps)
        q = np.stack([np.cos(a / 2), 0 * a, 0 * a, np.sin(a / 2)], 1)
    else:
        q = rng.normal(size=(n_clumps, 4))
        q /= np.linalg.norm(q, axis=1, keepdims=True)
    return pos_p, cid, q


def make_inputs(name, c):
    """Seeded inputs of one case (numpy PCG64)."""
    rng = np.random.Generator(np.random.PCG64(c["seed"]))
    N, dim = c["N"], c["dim"]
    if c["radii"] == "clump":
        return _clump_inputs(rng, c)
    if c["radii"] == "bi":
        rad = rng.choice([0.5, 0.7], size=N)
    elif c["radii"] == "poly":
        rad = rng.uniform(0.4, 0.6, size=N)
    else:
        rad = np.full(N, 0.5)
    rad = rad.astype(np.float32)
    vol = (np.pi * rad**2) if dim == 2 else (4.0 / 3.0 * np.pi * rad**3)
    L = c.get("box") or float((vol.astype(np.float64).sum() / c["phi"]) ** (1.0 / dim))
    if c["domain"] == "reflect":
        pos = rng.uniform(0, 1, size=(N, dim)) * (L - 2 * rad[:, None]) + rad[:, None]
    else:
        pos = rng.uniform(0.0, L, size=(N, dim))
    vel = rng.normal(0.0, c["vsig"], size=(N, dim))
    ad = 3 if dim == 3 else 1
    ang = rng.normal(0.0, c.get("wsig", 0.0), size=(N, ad)) if c.get("wsig") else np.zeros((N, ad))
    nmat = len(c.get("young", [1.0e3]))
    mat = rng.integers(0, nmat, size=N) if nmat > 1 else np.zeros(N, np.int64)
    return dict(pos=pos.astype(np.float32), vel=vel.astype(np.float32), rad=rad, ang_vel=ang.astype(np.float32),
                mat_id=mat.astype(np.int32), box=np.full(dim, L, np.float32), anchor=np.zeros(dim, np.float32))


def _clump_inputs(rng, c):
    """A clump case: ``N`` clumps; members carry their clump's centre, velocity, spin,
    orientation, mass (the members' volumes at density 1) and principal inertia."""
    dim, nc = c["dim"], c["N"]
    pos_p, cid, qc = _clumps(rng, nc, dim)
    N = len(cid)
    rad = rng.uniform(0.4, 0.5, N).astype(np.float32)
    vol = (np.pi * rad.astype(np.float64) ** 2) if dim == 2 else (4.0 / 3.0 * np.pi * rad.astype(np.float64) ** 3)
    L = float((vol.sum() / c["phi"]) ** (1.0 / dim))
    lo, hi = (1.0, L - 1.0) if c["domain"] == "reflect" else (0.0, L)
    centres = rng.uniform(lo, hi, (nc, dim))
    vc = rng.normal(0.0, c["vsig"], (nc, dim))
    ad = 3 if dim == 3 else 1
    wc = rng.normal(0.0, c["wsig"], (nc, ad))
    Mc = np.bincount(cid, weights=vol)
    Ic = np.stack([Mc * (0.2 + 0.05 * a) for a in range(ad)], 1)
    nmat = len(c.get("young", [1.0e3]))
    mat = rng.integers(0, nmat, size=N) if nmat > 1 else np.zeros(N, np.int64)
    f = np.float32
    return dict(pos=centres[cid].astype(f), vel=vc[cid].astype(f), rad=rad, ang_vel=wc[cid].astype(f),
                mat_id=mat.astype(np.int32), box=np.full(dim, L, f), anchor=np.zeros(dim, f),
                pos_p=pos_p.astype(f), q=qc[cid].astype(f), clump_id=cid.astype(np.int32), mass_in=Mc[cid].astype(f),
                inertia_in=Ic[cid].astype(f))


def _materials(jd, c):
    """The case's materials: "elastic" (young, Poisson 0.3), or "elasticfrict" with the
    case's poisson / e / mu / mu_r lists for the Cundall-Strack law."""
    youngs = c.get("young", [1.0e3])
    if c.get("law") == "cundallstrack":
        return [jd.Material.create("elasticfrict", density=1.0, young=float(y), poisson=float(p), mu=float(mu),
                                   e=float(e), mu_r=float(mr))
                for y, p, e, mu, mr in zip(youngs, c["poisson"], c["e"], c["mu"], c["mu_r"])]
    return [jd.Material.create("elastic", density=1.0, young=float(y), poisson=0.3) for y in youngs]


def run_case(jd, name, c, x64):
    import jax.numpy as jnp

    inp = make_inputs(name, c)
    dim = c["dim"]
    mat_table = jd.MaterialTable.from_materials(_materials(jd, c))
    fdt = np.float64 if x64 else np.float32
    if "clump_id" in inp:
        state = jd.State.create(pos=inp["pos"].astype(fdt), pos_p=inp["pos_p"].astype(fdt), q=inp["q"].astype(fdt),
                                vel=inp["vel"].astype(fdt), rad=inp["rad"].astype(fdt),
                                ang_vel=inp["ang_vel"].astype(fdt), mass=inp.pop("mass_in").astype(fdt),
                                inertia=inp.pop("inertia_in").astype(fdt), clump_id=inp["clump_id"],
                                mat_id=inp["mat_id"])
    else:
        state = jd.State.create(pos=inp["pos"].astype(fdt), vel=inp["vel"].astype(fdt), rad=inp["rad"].astype(fdt),
                                ang_vel=inp["ang_vel"].astype(fdt), mat_id=inp["mat_id"], mat_table=mat_table)
    domain_kw = {"box_size": tuple(float(x) for x in inp["box"]), "anchor": tuple(float(x) for x in inp["anchor"])}
    if c["domain"] == "reflect":
        domain_kw["restitution_coefficient"] = float(c.get("restitution", 1.0))
    fm_kw = {"gravity": c["gravity"]} if c.get("gravity") else None
    coll = c.get("collider", "CellList")
    coll_kw = {"state": state}
    if coll == "NeighborList":
        coll_kw.update(cutoff=2.0 * float(inp["rad"].max()), skin=float(c["nl_skin"]), max_neighbors=48)
    system = jd.System.create(
        state.shape, dt=c["dt"], domain_type=c["domain"], domain_kw=domain_kw, collider_type=coll,
        collider_kw=coll_kw, mat_table=mat_table, force_model_type=c.get("law", "spring"),
        linear_integrator_type=c.get("linear", "verlet"), rotation_integrator_type=c.get("rotation", "verletspiral"),
        force_manager_kw=fm_kw)
    out = {k: np.asarray(v) for k, v in inp.items()}
    out["mass"] = np.asarray(state.mass)
    out["inertia"] = np.asarray(state.inertia)
    out["young_eff"] = np.asarray(system.mat_table.young_eff)
    cl = system.collider.secondary_collider if coll == "NeighborList" else system.collider
    out["cell_size"] = np.asarray(cl.cell_size)
    # compute_force from the inputs (cell_list.py:434-464) and the energies (thermal.py:127-177)
    s0, sy0 = system.collider.compute_force(state, system)
    out["force0"] = np.asarray(s0.force)
    out["torque0"] = np.asarray(s0.torque)
    out["pe0"] = np.asarray(jd.utils.thermal.compute_potential_energy(state, system))
    out["ke0"] = np.asarray(jd.utils.thermal.compute_translational_kinetic_energy(state))
    out["kerot0"] = np.asarray(jd.utils.thermal.compute_rotational_kinetic_energy(state))
    if c.get("nl"):
        cutoff = float(c["nl"]) * float(inp["rad"].max())
        _, _, nl, ovf = system.collider.create_neighbor_list(state, system, cutoff, 48)
        out["nl_cutoff"] = np.float32(cutoff)
        out["nl"] = np.asarray(nl)
        out["nl_overflow"] = np.asarray(ovf)
    # snapshots after each stride of System.step
    st, sy = state, system
    snaps = {k: [] for k in ("pos", "vel", "force", "q", "ang_vel", "torque", "box", "anchor", "pe", "ke")}
    steps = 0
    for k in c["strides"]:
        st, sy = jd.System.step(st, sy, n=int(k))
        steps += int(k)
        snaps["pos"].append(np.asarray(st.pos_c))
        snaps["vel"].append(np.asarray(st.vel))
        snaps["force"].append(np.asarray(st.force))
        snaps["q"].append(np.asarray(jnp.stack([st.q.w[..., 0], st.q.xyz[..., 0], st.q.xyz[..., 1], st.q.xyz[..., 2]], -1)))
        snaps["ang_vel"].append(np.asarray(st.ang_vel))
        snaps["torque"].append(np.asarray(st.torque))
        snaps["box"].append(np.asarray(sy.domain.box_size))
        snaps["anchor"].append(np.asarray(sy.domain.anchor))
        snaps["pe"].append(np.asarray(jd.utils.thermal.compute_potential_energy(st, sy)))
        snaps["ke"].append(np.asarray(jd.utils.thermal.compute_translational_kinetic_energy(st)))
    for k, v in snaps.items():
        out["snap_" + k] = np.stack(v)
    if coll == "NeighborList":
        out["nl_builds"] = np.asarray(sy.collider.n_build_times)
        out["nl_max"] = np.asarray(system.collider.max_neighbors)
        out["nl_list_cutoff"] = np.asarray(system.collider.cutoff)
        out["nl_list_skin"] = np.asarray(system.collider.skin)
    out["snap_steps"] = np.cumsum(c["strides"]).astype(np.int32)
    out["meta"] = np.array(json.dumps({"case": name, "x64": x64, **c}))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--only", default=None)
    ap.add_argument("--x64", action="store_true", help="(internal) run the x64 variants in this process")
    a = ap.parse_args()
    sys.path.insert(0, str(HERE))
    import refenv

    jd = refenv.import_reference(a.reference, x64=a.x64)
    names = [a.only] if a.only else (X64_CASES if a.x64 else sorted(CASES))
    for name in names:
        t0 = time.time()
        out = run_case(jd, name, CASES[name], a.x64)
        path = HERE / f"reference_{name}{'_x64' if a.x64 else ''}.npz"
        np.savez_compressed(path, **out)
        print(f"{path.name}: {time.time() - t0:.1f} s", flush=True)
    if not a.x64 and not a.only:
        subprocess.run([sys.executable, __file__, "--reference", a.reference, "--x64"], check=True)


if __name__ == "__main__":
    main()
