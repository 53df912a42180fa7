"""Autotuner for the tracer's launch shape and grid density.

Searches the product of a small space exhaustively -- cells per triangle k,
ray tile order (scanline / Morton 8x8), empty-cell run length, persistent vs
one-shot trace grid, the list length above which a ray is finished by the
warp-per-ray pass, cell-ordered triangle records, lane refill -- timing each candidate with a caller-supplied
measurement (CUDA events on the scene's stream), and caches the winner in a
JSON file keyed by a workload signature (triangles, rays, scene box extent),
so a second run of the same workload skips the search.  None of these
parameters changes a result: the grid and the hits are identical for every
choice except k, which defines the grid (and is part of the signature when
the caller fixes it).
"""
from __future__ import annotations

import itertools
import json
import os
import time
from typing import Callable, Dict, Iterable, List, Tuple

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "tune_cache.json")

SPACE = {
    "order": ("scanline", "morton8"),
    "empty_run": (2, 4, 8),
    "persistent": (True, False),
    "heavy_cell": (0, 24, 32, 48),
    "heavy_lanes": (16, 32),
    "cell_records": (False, True),
    "refill": (0, 16),
}


def _load() -> dict:
    try:
        with open(CACHE) as f:
            return json.load(f)
    except Exception:
        return {}


def _store(d: dict) -> None:
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + f".{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def signature(**kw) -> str:
    return ",".join(f"{k}={kw[k]}" for k in sorted(kw))


def search(measure: Callable[[dict], float], space: Dict[str, Iterable] = None, key: str = None,
           reps: int = 3, use_cache: bool = True) -> Tuple[dict, List[Tuple[dict, float]]]:
    """Exhaustive search; measure(cfg) -> milliseconds (lower is better).
    Each candidate is measured `reps` times and scored by its minimum."""
    space = dict(space or SPACE)
    cache = _load() if (use_cache and key) else {}
    if key and key in cache:
        return cache[key]["best"], [(c["cfg"], c["ms"]) for c in cache[key]["all"]]
    names = sorted(space)
    results = []
    for values in itertools.product(*(tuple(space[n]) for n in names)):
        cfg = dict(zip(names, values))
        ms = min(measure(cfg) for _ in range(reps))
        results.append((cfg, ms))
    best = min(results, key=lambda r: r[1])[0]
    if key:
        cache = _load()
        cache[key] = {"best": best, "all": [{"cfg": c, "ms": m} for c, m in results], "when": time.time()}
        _store(cache)
    return best, results
