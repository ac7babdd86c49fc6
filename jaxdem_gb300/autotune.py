"""Autotuner for the engine's tunable shapes.

* skin: list length (pair tests every step grow as (2r + skin)^3) against the
  re-sort rate (a re-sort is due when the accumulated displacement reaches
  skin / 2);
* prune skin: the inner list of the dynamic pruning, shorter with a small
  margin but rebuilt from the full list more often (off, or a fraction of the
  skin);
* brick size: particles per shared-memory brick of the list build (larger
  bricks stage relatively fewer halo cells but fill fewer blocks);
* force-kernel shape: threads per block of the fused force kernel above
  32768 particles (64, 128 or 256: how many slots retire together against
  the block-granular residency), or, at most 32768 particles, lanes sharing a
  slot in the per-step and many-step force kernels (4, 8 or 16: a slot's row
  split across more lanes shortens its chain of dependent loads but occupies
  more threads and shuffles more partial sums).

The best values depend on density, temperature and size, so they are
measured: a coordinate search times a short chunk of steps on the actual
system for each candidate of one shape at a time (skin, then prune skin, then
brick size, then the force-kernel shape), keeping the fastest.  Results are cached per configuration class
(dimension, log2 particle bucket, density bucket, mean speed bucket) in a JSON
file, so repeated runs of similar workloads skip the search.
"""

from __future__ import annotations

import json
import math
import os
import time
from pathlib import Path
from typing import Callable, Optional, Sequence

import numpy as np

# in units of r_max; the large skins pay off for small systems, whose steps
# cost little next to a re-sort (many-step launches)
CANDIDATES = (0.15, 0.3, 0.45, 0.65, 0.9, 1.2, 1.6, 2.0)
CACHE = Path(os.environ.get("JDEM_TUNE_CACHE", Path.home() / ".cache" / "jaxdem_gb300" / "tune.json"))


def default_skin(rmax: float) -> float:
    """Skin used without tuning: 0.65 r_max (near the optimum measured on the dense 3D benchmark)."""
    return 0.65 * float(rmax)


def config_key(dim: int, n: int, phi: float, vrms: float, domain: str) -> str:
    nb = int(round(math.log2(max(n, 1))))
    pb = int(round(phi * 20))
    vb = int(round(math.log2(max(vrms, 1e-6))))
    return f"{dim}d-{domain}-n{nb}-phi{pb}-v{vb}"


def _load() -> dict:
    try:
        return json.loads(CACHE.read_text())
    except Exception:
        return {}


def _store(d: dict) -> None:
    try:
        CACHE.parent.mkdir(parents=True, exist_ok=True)
        CACHE.write_text(json.dumps(d, indent=1, sort_keys=True))
    except OSError:
        pass


def workload_key(w) -> str:
    from .workloads import volume

    vol = float(np.prod(np.asarray(w.box_size, np.float64)))
    phi = float(volume(w.rad, w.dim).astype(np.float64).sum() / vol) if vol > 0 else 0.0
    vrms = float(np.sqrt(np.mean(np.asarray(w.vel, np.float64) ** 2))) if w.N else 0.0
    return config_key(w.dim, w.N, phi, vrms, w.domain)


# prune skin as a fraction of the skin (-1: pruning off), list-build brick sizes,
# force-kernel block sizes (above 32768 particles) and lanes per slot and brick sizes
# (at most 32768: few particles make few bricks, so smaller ones keep more SMs busy)
PRUNE_CANDIDATES = (-1.0, 0.2, 1.0 / 3.0, 0.5)
BRICK_CANDIDATES = (120, 240, 480)
SMALL_BRICK_CANDIDATES = (30, 60, 120)
BLOCK_CANDIDATES = (64, 128, 256)
LANE_CANDIDATES = (4, 8, 16)
SMALL_SLOTS = 32768


def _time_chunk(make_engine, upload, params, steps):
    eng = make_engine(**params)
    try:
        upload(eng)
        # warm-up with the timed call itself: the first re-sort, and every CUDA graph the
        # timed call launches is captured before the clock starts
        eng.step(steps)
        eng.sync()
        t0 = time.perf_counter()
        eng.step(steps)
        return (time.perf_counter() - t0) / steps
    finally:
        eng.close()


def tune_shapes(make_engine: Callable[..., "object"], upload: Callable[["object"], None], rmax: float,
                n_particles: int, key: Optional[str] = None, steps: int = 60, use_cache: bool = True) -> tuple[dict, dict]:
    """Coordinate search over (skin, prune skin, brick size, force-kernel shape); returns (best, timings).

    ``make_engine(skin=..., prune_skin=..., brick_particles=..., force_block=..., small_lanes=...)``
    builds an engine and ``upload(engine)`` loads the state.  ``best`` holds those five
    arguments; ``timings`` the seconds per step of every candidate, per shape.  The prune
    skin and block size only matter above 32768 particles (the fused list kernel); at most
    32768 particles the skin, the lanes per slot and the (smaller) brick sizes are tuned.
    """
    cache = _load() if use_cache else {}
    ckey = None if key is None else "shapes:" + key
    if ckey is not None and ckey in cache:
        c = cache[ckey]
        return ({"skin": c["skin_rel"] * rmax, "prune_skin": c["prune_rel"] * c["skin_rel"] * rmax
                 if c["prune_rel"] > 0 else -1.0, "brick_particles": int(c["brick"]),
                 "force_block": int(c.get("block", 128)), "small_lanes": int(c.get("lanes", 8))},
                c.get("timings", {}))
    timings = {"skin": {}, "prune": {}, "brick": {}, "block": {}, "lanes": {}}
    large = n_particles > SMALL_SLOTS
    cur = {"prune_skin": 0.0, "brick_particles": 240 if large else 60, "force_block": 128, "small_lanes": 8}
    for c in CANDIDATES:
        timings["skin"][str(c)] = _time_chunk(make_engine, upload, {**cur, "skin": c * rmax}, steps)
    skin_rel = float(min(timings["skin"], key=timings["skin"].get))
    cur["skin"] = skin_rel * rmax
    prune_rel = 1.0 / 3.0
    if large:
        for pr in PRUNE_CANDIDATES:
            ps = -1.0 if pr < 0 else pr * cur["skin"]
            timings["prune"][str(round(pr, 3))] = _time_chunk(make_engine, upload, {**cur, "prune_skin": ps}, steps)
        prune_rel = float(min(timings["prune"], key=timings["prune"].get))
        cur["prune_skin"] = -1.0 if prune_rel < 0 else prune_rel * cur["skin"]
        for bk in BRICK_CANDIDATES:
            timings["brick"][str(bk)] = _time_chunk(make_engine, upload, {**cur, "brick_particles": bk}, steps)
        cur["brick_particles"] = int(min(timings["brick"], key=timings["brick"].get))
        for nt in BLOCK_CANDIDATES:
            timings["block"][str(nt)] = _time_chunk(make_engine, upload, {**cur, "force_block": nt}, steps)
        cur["force_block"] = int(min(timings["block"], key=timings["block"].get))
    else:
        for g in LANE_CANDIDATES:
            timings["lanes"][str(g)] = _time_chunk(make_engine, upload, {**cur, "small_lanes": g}, steps)
        cur["small_lanes"] = int(min(timings["lanes"], key=timings["lanes"].get))
        for bk in SMALL_BRICK_CANDIDATES:
            timings["brick"][str(bk)] = _time_chunk(make_engine, upload, {**cur, "brick_particles": bk}, steps)
        cur["brick_particles"] = int(min(timings["brick"], key=timings["brick"].get))
    best = {"skin": cur["skin"], "prune_skin": -1.0 if prune_rel < 0 else prune_rel * cur["skin"],
            "brick_particles": cur["brick_particles"], "force_block": cur["force_block"],
            "small_lanes": cur["small_lanes"]}
    if ckey is not None:
        cache[ckey] = {"skin_rel": skin_rel, "prune_rel": prune_rel, "brick": cur["brick_particles"],
                       "block": cur["force_block"], "lanes": cur["small_lanes"], "timings": timings}
        _store(cache)
    return best, timings
