"""The engine, through the C ABI, against golden vectors produced by JaxDEM's own code
(tests/golden/reference_<case>.npz; see tests/golden/make_reference_golden.py).

Bars of the benchmark specification: forces within 1e-5 floored relative error of the
reference's float32 compute_force (torques within 1e-5 of the largest torque); positions
within 1e-4 after each recorded stride of System.step; rotation state (q, ang_vel) for the
VV-spiral and spiral integrators; the reference's create_neighbor_list bit for bit; energies
within 1e-5.  The cases include the Cundall-Strack law (rolling friction, two materials) and
rigid clumps, in periodic and reflecting boxes.  Against the float64
(jax_enable_x64) runs the float32 engine's error is stated and bounded.
"""

from __future__ import annotations

import numpy as np
import pytest

from jaxdem_gb300._lib import Engine
from tests.helpers import (force_err, global_force_err, load_reference_case, min_image_diff,
                           reference_case_names, reference_osystem)

pytestmark = pytest.mark.gpu

CASES = reference_case_names()


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def _engine(d):
    m = d["meta"]
    sy = reference_osystem(d)
    desc = dict(n=len(d["pos"]), domain=m["domain"], linear=m.get("linear", "verlet"),
                rotation=m.get("rotation", "verletspiral"), dt=m["dt"], box_size=d["box"], anchor=d["anchor"],
                restitution=m.get("restitution", 1.0), gravity=sy.gravity, cell_size=float(d["cell_size"]),
                search_range=1)
    return Engine(m["dim"], [desc], sy.young_eff, skin=0.1 * float(d["rad"].max()),
                  force_law=m.get("law", "spring"), material_props=sy.mat_props)


def _upload(eng, d):
    clump = {k: d[k] for k in ("pos_p", "q", "clump_id") if k in d}
    eng.upload(pos=d["pos"], vel=d["vel"], rad=d["rad"], mass=d["mass"], mat_id=d["mat_id"], ang_vel=d["ang_vel"],
               inertia=d["inertia"], **clump)


def _torque_err(t, ref):
    """Largest torque error over the largest reference torque (torques are zero for
    smooth spheres under the central spring and Hertz laws)."""
    scale = max(float(np.abs(ref).max()), 1e-30)
    return float(np.abs(t - ref).max()) / scale


@pytest.mark.parametrize("name", CASES)
def test_engine_matches_reference_outputs(name):
    d = load_reference_case(name)
    box = d["box"] if d["meta"]["domain"] == "periodic" else None
    eng = _engine(d)
    try:
        _upload(eng, d)
        e0 = eng.energy()
        eng.compute_force()
        out0 = eng.download()
        f0 = out0["force"]
        _upload(eng, d)
        prev, snaps = 0, []
        for n in d["snap_steps"]:
            eng.step(int(n - prev))
            prev = n
            snaps.append(eng.download())
        nl = None
        if "nl" in d:
            _upload(eng, d)
            nl, ovf = eng.neighbor_list(float(d["nl_cutoff"]), int(d["nl"].shape[1]))
    finally:
        eng.close()
    assert force_err(f0, d["force0"]) <= 1e-5, f"{name}: compute_force err {force_err(f0, d['force0'])}"
    assert global_force_err(f0, d["force0"]) <= 1e-5
    assert _torque_err(out0["torque"], d["torque0"]) <= 1e-5, f"{name}: torque err"
    # thermal.compute_potential_energy: force-manager (gravity) PE + collider PE
    assert np.allclose(e0[0] + e0[1], d["pe0"], rtol=1e-5, atol=1e-5), (e0, d["pe0"])
    assert np.allclose(e0[2], d["ke0"], rtol=1e-5, atol=1e-6)
    for i, out in enumerate(snaps):
        n = int(d["snap_steps"][i])
        dp = min_image_diff(out["pos_c"], d["snap_pos"][i], box)
        assert dp <= 1e-4, f"{name} after {n} steps: position error {dp}"
        assert np.abs(out["vel"] - d["snap_vel"][i]).max() <= 1e-4 * max(1.0, np.abs(d["snap_vel"][i]).max())
        assert force_err(out["force"], d["snap_force"][i]) <= 1e-4
        assert np.allclose(out["q"], d["snap_q"][i], atol=2e-6), f"{name}: q after {n} steps"
        assert np.allclose(out["ang_vel"], d["snap_ang_vel"][i], rtol=1e-5, atol=1e-5)
        assert _torque_err(out["torque"], d["snap_torque"][i]) <= 1e-4, f"{name}: torque after {n} steps"
    if nl is not None:
        assert ovf == bool(d["nl_overflow"])
        assert np.array_equal(nl, d["nl"])


@pytest.mark.parametrize("name", ["per3d_bi", "refl2d_grav"])
def test_engine_error_against_reference_x64(name):
    """The float32 engine against the reference run in float64: the stated error."""
    d = load_reference_case(name, x64=True)
    box = d["box"] if d["meta"]["domain"] == "periodic" else None
    eng = _engine(d)
    try:
        _upload(eng, d)
        eng.compute_force()
        f0 = eng.download()["force"]
        _upload(eng, d)
        eng.step(int(d["snap_steps"][-1]))
        out = eng.download()
    finally:
        eng.close()
    ef = force_err(f0, d["force0"])
    dp = min_image_diff(out["pos_c"], d["snap_pos"][-1], box)
    print(f"{name}: float32 engine vs float64 reference: force err {ef:.2e}, position err {dp:.2e} "
          f"after {int(d['snap_steps'][-1])} steps")
    assert ef <= 1e-5
    assert dp <= 1e-4
