"""Autotuner for the engine's tunable shape: the binning/list skin.

The skin trades list length (pair tests every step grow as (2r + skin)^3)
against the re-sort rate (a re-sort is due when the accumulated displacement
reaches skin / 2).  The best value depends on density, temperature and size,
so it is measured: a few candidate skins each run a short timed chunk on the
actual system, and the fastest wins.  Results are cached per configuration
class (dimension, log2 particle bucket, density bucket, mean speed bucket)
in a JSON file, so repeated runs of similar workloads skip the search.
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


def tune_skin(make_engine: Callable[[float], "object"], upload: Callable[["object"], None], rmax: float,
              key: Optional[str] = None, steps: int = 60, candidates: Sequence[float] = CANDIDATES,
              use_cache: bool = True) -> tuple[float, dict]:
    """Return (best skin, {skin: seconds per step}).

    ``make_engine(skin)`` builds an engine, ``upload(engine)`` loads the
    state; each candidate runs ``steps`` steps after a warm-up chunk.
    """
    cache = _load() if use_cache else {}
    if key is not None and key in cache:
        return float(cache[key]["skin_rel"]) * rmax, cache[key].get("timings", {})
    timings = {}
    for c in candidates:
        skin = c * rmax
        eng = make_engine(skin)
        try:
            upload(eng)
            eng.step(max(10, steps // 3))  # warm-up: first re-sort, graph capture
            eng.sync()
            t0 = time.perf_counter()
            eng.step(steps)
            timings[c] = (time.perf_counter() - t0) / steps
        finally:
            eng.close()
    best = min(timings, key=timings.get)
    if key is not None:
        cache[key] = {"skin_rel": best, "timings": {str(k): v for k, v in timings.items()}}
        _store(cache)
    return best * rmax, timings


def workload_key(w) -> str:
    from .workloads import volume

    vol = float(np.prod(np.asarray(w.box_size, np.float64)))
    phi = float(volume(w.rad, w.dim).astype(np.float64).sum() / vol) if vol > 0 else 0.0
    vrms = float(np.sqrt(np.mean(np.asarray(w.vel, np.float64) ** 2))) if w.N else 0.0
    return config_key(w.dim, w.N, phi, vrms, w.domain)
