"""The shape autotuner's coordinate search and cache (host logic; timings are synthetic)."""

from __future__ import annotations

import json

from jaxdem_gb300 import autotune


def test_coordinate_search_picks_each_shape_and_caches(monkeypatch, tmp_path):
    calls = []

    def fake_time(make_engine, upload, params, steps):
        calls.append(dict(params))
        skin, ps, bk = params["skin"], params["prune_skin"], params["brick_particles"]
        cost = (skin - 0.455) ** 2 + 0.1
        if ps > 0:
            cost -= 0.02 * (1.0 - abs(ps / skin - 0.2))  # pruning at 0.2 x skin is best
        cost += 0.001 * abs(bk - 480) / 480
        cost += 0.0005 * (params["force_block"] != 64)
        assert params["small_lanes"] == 8  # not tuned above 32768 particles
        return cost

    monkeypatch.setattr(autotune, "_time_chunk", fake_time)
    monkeypatch.setattr(autotune, "CACHE", tmp_path / "tune.json")
    best, timings = autotune.tune_shapes(None, None, 0.7, 1 << 20, key="k")
    assert abs(best["skin"] - 0.65 * 0.7) < 1e-9
    assert abs(best["prune_skin"] - 0.2 * best["skin"]) < 1e-9
    assert best["brick_particles"] == 480
    assert best["force_block"] == 64 and best["small_lanes"] == 8
    n = len(calls)
    assert n == (len(autotune.CANDIDATES) + len(autotune.PRUNE_CANDIDATES) + len(autotune.BRICK_CANDIDATES)
                 + len(autotune.BLOCK_CANDIDATES))
    # each shape is searched with the best values found before it
    assert all(c["brick_particles"] == 480 for c in calls[-len(autotune.BLOCK_CANDIDATES):])
    assert set(timings) == {"skin", "prune", "brick", "block", "lanes"} and timings["lanes"] == {}
    cached = json.loads((tmp_path / "tune.json").read_text())["shapes:k"]
    assert cached["brick"] == 480 and cached["block"] == 64
    # a second call is served from the cache
    best2, _ = autotune.tune_shapes(None, None, 0.7, 1 << 20, key="k")
    assert len(calls) == n and best2 == best


def test_small_systems_tune_the_skin_lanes_per_slot_and_bricks(monkeypatch, tmp_path):
    seen = []
    monkeypatch.setattr(autotune, "_time_chunk",
                        lambda mk, up, p, s: seen.append(p) or p["skin"] + 0.001 * abs(p["small_lanes"] - 16)
                        + 1e-6 * abs(p["brick_particles"] - 30))
    monkeypatch.setattr(autotune, "CACHE", tmp_path / "tune.json")
    best, timings = autotune.tune_shapes(None, None, 0.5, 4096, key=None)
    n_lanes, n_bricks = len(autotune.LANE_CANDIDATES), len(autotune.SMALL_BRICK_CANDIDATES)
    assert len(seen) == len(autotune.CANDIDATES) + n_lanes + n_bricks
    assert best["skin"] == min(autotune.CANDIDATES) * 0.5 and timings["prune"] == {} and timings["block"] == {}
    assert best["small_lanes"] == 16 and best["force_block"] == 128 and best["brick_particles"] == 30
    assert all(p["brick_particles"] == 60 for p in seen[:-n_bricks])  # the small-handle default until tuned
    assert all(p["skin"] == best["skin"] for p in seen[-(n_lanes + n_bricks):])
    assert all(p["small_lanes"] == 16 for p in seen[-n_bricks:])


def test_batch_tune_key_separates_batches():
    from jaxdem_gb300 import workloads as W
    from jaxdem_gb300.batch import tune_key

    a, b = W.c4(n_systems=16, seed=4), W.c4(n_systems=32, seed=4)
    assert tune_key(a) == tune_key(W.c4(n_systems=16, seed=4))
    assert tune_key(a) != tune_key(b) and tune_key(a).startswith("batch16-3d-periodic-")
