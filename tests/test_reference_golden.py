"""The oracle pinned against golden vectors produced by JaxDEM's own code.

tests/golden/reference_<case>.npz were written by tests/golden/make_reference_golden.py,
which runs the reference's source (State.create, System.create, System.step,
DynamicCellList.compute_force / create_neighbor_list, the thermal energies) on a numpy
stand-in for the JAX API.  The numpy restatement (oracle/dem_ref.py) follows the
reference's float32 operation order, so it must reproduce those outputs bit for bit; the C
restatement (oracle/jdem_oracle.c, the fast oracle the GPU tests use) must too, for the
cases it covers (spring and Hertz laws, Verlet and Euler, periodic / reflect / free).  The
float64 cases (jax_enable_x64) pin the oracle's float64 build.

Cases: 3D bidisperse periodic, 2D polydisperse periodic, 2D reflect with gravity, 3D
reflect with restitution 0.8 and gravity, 3D free domain, VV-spiral and spiral rotation
with random spins, Hertz law, two materials, direct Euler, a periodic box of two cells
per axis (the reference de-duplicates the stencil), Cundall-Strack with two "elasticfrict"
materials and rolling friction (3D periodic; 2D reflect with gravity and the spiral
integrator), rigid clumps of one to three spheres (3D periodic; 2D reflect with gravity), with
and without Cundall-Strack contacts, and the NeighborList collider (cached list with skin,
rebuilt on displacement; 3D periodic, 2D reflect with gravity).

One reduction is not bit-reproducible by construction: the reference sums each particle's
per-stencil-cell accumulators with ``x.sum(axis=0)`` (``colliders/cell_list.py:255-256``),
whose order XLA leaves unspecified.  On the numpy stand-in that sum is pairwise over the
contiguous (9, 1) torque block of a 2D particle (numpy's 8-way blocked summation), where the
oracle adds the nine cells left to right.  Only 2D torques that are non-zero and spread over
at least eight cells see it (the 2D Cundall-Strack case): there the torque, the angular
velocity and the orientation are held to a few float32 ulps, everything else bit for bit.
"""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from oracle import dem_ref as R
from tests.helpers import (force_err, load_reference_case, min_image_diff, reference_case_names,
                           reference_osystem, reference_ostate)

CASES = reference_case_names()
X64_CASES = ["per3d_bi", "refl2d_grav"]


def test_fixture_set_is_complete():
    assert len(CASES) >= 19, CASES
    laws = {load_reference_case(c)["meta"].get("law", "spring") for c in CASES}
    assert laws == {"spring", "hertz", "cundallstrack"}
    assert sum("clump_id" in load_reference_case(c) for c in CASES) >= 2


def _torque_order_free(d):
    """2D cases with pair torques: the stencil-cell sum order of the torque is unspecified."""
    return d["meta"]["dim"] == 2 and d["meta"].get("law") == "cundallstrack"


def _same(a, b, loose, rtol=1e-6, atol=0.0):
    return np.allclose(a, b, rtol=rtol, atol=atol) if loose else np.array_equal(a, b)


@pytest.mark.parametrize("name", CASES)
def test_numpy_oracle_reproduces_reference_bit_for_bit(name):
    d = load_reference_case(name)
    loose = _torque_order_free(d)
    st = reference_ostate(d)
    f0, t0 = R.collider_force(st, reference_osystem(d))
    sy = reference_osystem(d)
    assert np.array_equal(f0, d["force0"]), f"{name}: compute_force differs (err {force_err(f0, d['force0'])})"
    assert _same(t0, d["torque0"], loose, atol=1e-6 * np.abs(d["torque0"]).max())
    e = R.compute_energy(st, sy)
    # thermal.compute_potential_energy: force-manager (gravity) PE + collider PE
    assert np.isclose(e[0] + e[1], d["pe0"], rtol=1e-6, atol=1e-6)
    assert np.isclose(e[2], d["ke0"], rtol=1e-6, atol=1e-7)
    s, prev = st.copy(), 0
    box = d["box"] if d["meta"]["domain"] == "periodic" else None
    for i, n in enumerate(d["snap_steps"]):
        s, sy = R.step(s, sy, int(n - prev))
        prev = n
        assert np.array_equal(s.pos_c, d["snap_pos"][i]), (
            f"{name} after {n} steps: positions differ by {min_image_diff(s.pos_c, d['snap_pos'][i], box)}")
        assert np.array_equal(s.vel, d["snap_vel"][i])
        assert np.array_equal(s.force, d["snap_force"][i])
        assert _same(s.q, d["snap_q"][i], loose, rtol=0.0, atol=1e-7)
        assert _same(s.ang_vel, d["snap_ang_vel"][i], loose, atol=1e-6)
        assert _same(s.torque, d["snap_torque"][i], loose, atol=1e-6 * np.abs(d["snap_torque"][i]).max())
        if d["meta"]["domain"] == "free":
            assert np.array_equal(sy.box_size, d["snap_box"][i])
            assert np.array_equal(sy.anchor, d["snap_anchor"][i])


@pytest.mark.parametrize("name", [c for c in CASES if "nl" in load_reference_case(c)])
def test_neighbor_list_reproduces_reference(name):
    d = load_reference_case(name)
    sy, st = reference_osystem(d), reference_ostate(d)
    nl, ovf = R.create_neighbor_list(st, sy, float(d["nl_cutoff"]), int(d["nl"].shape[1]))
    assert bool(ovf) == bool(d["nl_overflow"])
    assert np.array_equal(nl, d["nl"])


def _c_covers(d):
    """The C restatement covers smooth spheres under the spring and Hertz laws with the
    cell-list collider."""
    return (not np.any(d["ang_vel"]) and "clump_id" not in d
            and d["meta"].get("law", "spring") in ("spring", "hertz")
            and d["meta"].get("collider", "CellList") == "CellList")


C_CASES = [c for c in CASES if _c_covers(load_reference_case(c))]


@pytest.mark.parametrize("name", C_CASES)
def test_c_oracle_reproduces_reference(name):
    d = load_reference_case(name)
    m = d["meta"]
    law = m.get("law", "spring")
    sy = reference_osystem(d)
    kw = dict(domain=m["domain"], box=d["box"], anchor=d["anchor"], cell_size=float(d["cell_size"]),
              young=sy.young_eff, mat_id=d["mat_id"], law=law)
    f0 = oracle.c_force(m["dim"], d["pos"], d["rad"], **kw)
    pos, vel, frc = d["pos"].copy(), d["vel"].copy(), np.zeros_like(d["pos"])
    box = d["box"] if m["domain"] == "periodic" else None
    if law == "hertz":
        # delta^(3/2): C's powf and numpy's float32 power may differ in the last bit
        assert force_err(f0, d["force0"]) <= 1e-6
    else:
        assert np.array_equal(f0, d["force0"]), f"{name}: C compute_force err {force_err(f0, d['force0'])}"
    prev = 0
    for i, n in enumerate(d["snap_steps"]):
        oracle.c_step(m["dim"], pos, vel, frc, d["rad"], d["mass"], dt=m["dt"], steps=int(n - prev),
                      gravity=m.get("gravity"), restitution=m.get("restitution", 1.0),
                      linear=m.get("linear", "verlet"), **kw)
        prev = n
        if law == "hertz":
            assert min_image_diff(pos, d["snap_pos"][i], box) <= 1e-6, f"{name} after {n} steps"
            assert force_err(frc, d["snap_force"][i]) <= 1e-5
            continue
        assert np.array_equal(pos, d["snap_pos"][i]), f"{name} after {n} steps"
        assert np.array_equal(vel, d["snap_vel"][i])
        assert np.array_equal(frc, d["snap_force"][i])


@pytest.mark.parametrize("name", X64_CASES)
def test_float64_oracle_reproduces_reference_x64(name):
    d = load_reference_case(name, x64=True)
    assert d["pos"].dtype == np.float32 and d["force0"].dtype == np.float64
    sy, st = reference_osystem(d, np.float64), reference_ostate(d, np.float64)
    f0, _ = R.cell_list_force(st, sy)
    assert force_err(f0, d["force0"]) <= 1e-13
    s, prev = st.copy(), 0
    for i, n in enumerate(d["snap_steps"]):
        s, sy = R.step(s, sy, int(n - prev))
        prev = n
        assert np.abs(s.pos_c - d["snap_pos"][i]).max() <= 1e-12, f"{name} after {n} steps"
        assert np.abs(s.vel - d["snap_vel"][i]).max() <= 1e-10
