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
        return cost

    monkeypatch.setattr(autotune, "_time_chunk", fake_time)
    monkeypatch.setattr(autotune, "CACHE", tmp_path / "tune.json")
    best, timings = autotune.tune_shapes(None, None, 0.7, 1 << 20, key="k")
    assert abs(best["skin"] - 0.65 * 0.7) < 1e-9
    assert abs(best["prune_skin"] - 0.2 * best["skin"]) < 1e-9
    assert best["brick_particles"] == 480
    n = len(calls)
    assert n == len(autotune.CANDIDATES) + len(autotune.PRUNE_CANDIDATES) + len(autotune.BRICK_CANDIDATES)
    assert set(timings) == {"skin", "prune", "brick"}
    cached = json.loads((tmp_path / "tune.json").read_text())["shapes:k"]
    assert cached["brick"] == 480
    # a second call is served from the cache
    best2, _ = autotune.tune_shapes(None, None, 0.7, 1 << 20, key="k")
    assert len(calls) == n and best2 == best


def test_small_systems_tune_the_skin_only(monkeypatch, tmp_path):
    seen = []
    monkeypatch.setattr(autotune, "_time_chunk", lambda mk, up, p, s: seen.append(p) or p["skin"])
    monkeypatch.setattr(autotune, "CACHE", tmp_path / "tune.json")
    best, timings = autotune.tune_shapes(None, None, 0.5, 4096, key=None)
    assert len(seen) == len(autotune.CANDIDATES)
    assert best["skin"] == min(autotune.CANDIDATES) * 0.5 and timings["prune"] == {}
