"""Force-kernel shapes the autotuner picks (JdemConfig.force_block, small_lanes).

* Threads per block of the fused force kernel (64, 128, 256) change nothing a
  thread computes, so trajectories are bit-identical across block shapes.
* Lanes per slot of the small-system kernels (4, 8, 16) regroup a slot's
  compensated partial sums; for each lane count the many-step kernel and the
  launch-per-step kernel still agree bit for bit, and the lane counts agree
  with each other and with the oracle at the force bar.
* Other values are rejected at create.
"""

from __future__ import annotations

import numpy as np
import pytest

from jaxdem_gb300 import workloads as W
from jaxdem_gb300._lib import Engine, JdemError
from oracle import dem_ref as R
from tests.helpers import force_err, min_image_diff, osystem, ostate

pytestmark = pytest.mark.gpu

K = np.array([[W.K_SPRING]], np.float32)


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def run(w, steps, **kw):
    eng = Engine(w.dim, [w.desc()], K, chunk_steps=25, **kw)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.step(steps)
        out = eng.download()
        st = eng.stats()
    finally:
        eng.close()
    return out, st


@pytest.mark.parametrize("block", [64, 256])
def test_force_block_shapes_are_bit_identical(block):
    w = W.c2(N=65536, seed=17)
    ref, sr = run(w, 60, skin=0.455, force_block=128)
    out, so = run(w, 60, skin=0.455, force_block=block)
    assert sr["rebuilds"] == so["rebuilds"] and sr["prunes"] == so["prunes"] and sr["prunes"] > 0
    for k in ("pos_c", "vel", "force"):
        assert np.array_equal(ref[k], out[k]), k


@pytest.mark.parametrize("lanes", [4, 8, 16])
def test_small_lanes_many_step_equals_per_step(lanes):
    w = W.c1(N=4096, seed=23)
    a, sa = run(w, 120, skin=0.2, small_lanes=lanes, graph_mode=0)
    b, sb = run(w, 120, skin=0.2, small_lanes=lanes, graph_mode=2)
    assert sa["many_step"] == 1 and sb["many_step"] == 0 and sa["rebuilds"] == sb["rebuilds"]
    for k in ("pos_c", "vel", "force"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("lanes", [4, 16])
def test_small_lanes_match_the_oracle(lanes):
    w = W.c2(N=8192, seed=29)
    out, _ = run(w, 1, skin=0.3, small_lanes=lanes, graph_mode=2)
    st1, _ = R.step(ostate(w), osystem(w), 1, sum_dtype=np.float64)
    assert force_err(out["force"], st1.force) <= 1e-5
    assert min_image_diff(out["pos_c"], st1.pos_c, w.box_size) <= 1e-5
    ref, _ = run(w, 40, skin=0.3, small_lanes=8, graph_mode=2)
    got, _ = run(w, 40, skin=0.3, small_lanes=lanes, graph_mode=2)
    assert min_image_diff(got["pos_c"], ref["pos_c"], w.box_size) <= 1e-5


@pytest.mark.parametrize("kw", [{"force_block": 96}, {"small_lanes": 2}, {"small_lanes": 32}])
def test_other_shapes_are_rejected(kw, capfd):
    w = W.c1(N=256, seed=3)
    with pytest.raises(JdemError) as ei:
        Engine(w.dim, [w.desc()], K, skin=0.2, **kw)
    assert ei.value.code == 1  # JDEM_ERR_BAD_ARG
    assert next(iter(kw)) in capfd.readouterr().err  # create reports on stderr (no handle yet)
