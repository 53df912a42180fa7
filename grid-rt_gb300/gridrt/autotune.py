"""Autotuner for the tracer's launch shape and grid density.

The space: cells per triangle k (when the caller lets it vary), ray tile
order (scanline / Morton 8x8), empty-cell run length, persistent vs one-shot
trace grid, threads per block of the one-lane trace launch, lanes per ray
from the start (one, or a group of 2 or 4 for every ray), the list length
above which a ray is finished by the warp-per-ray pass and that pass's lanes
per ray, cell-ordered triangle records, lane refill.  Each candidate is timed
with a caller-supplied measurement (CUDA events on the scene's stream).
Spaces of up to `exhaustive_max` candidates are searched exhaustively; larger
ones by coordinate descent -- from the first value of every dimension, each
dimension in turn is set to its best value with the others fixed, until a
full sweep changes nothing (at most `sweeps` sweeps) -- which times a few
dozen candidates instead of every product.  The winner can be cached in a
JSON file keyed by a workload signature, so a second run of the same
workload skips the search; the result says whether it came from the cache.
None of these parameters changes a result: the grid and the hits are
identical for every choice except k, which defines the grid.
"""
from __future__ import annotations

import itertools
import json
import os
import time
from typing import Callable, Dict, Iterable, List, Tuple

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "tune_cache.json")

SPACE = {
    "order": ("morton8", "scanline"),
    "empty_run": (4, 2, 8),
    "persistent": (True, False),
    "block": (128, 64, 256),
    "lanes": (1, 2, 4),
    "heavy_cell": (32, 0, 24, 48),
    "heavy_lanes": (32, 16),
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


def size(space: Dict[str, Iterable]) -> int:
    n = 1
    for v in space.values():
        n *= len(tuple(v))
    return n


def search(measure: Callable[[dict], float], space: Dict[str, Iterable] = None, key: str = None,
           reps: int = 3, use_cache: bool = True, exhaustive_max: int = 256,
           sweeps: int = 3) -> Tuple[dict, List[Tuple[dict, float]]]:
    """measure(cfg) -> milliseconds (lower is better); each candidate is
    measured `reps` times and scored by its minimum.  Returns (best, table)
    where table lists every timed candidate; search.last_source is "cache"
    or "search" for the last call."""
    space = {n: tuple(v) for n, v in (space or SPACE).items()}
    cache = _load() if (use_cache and key) else {}
    if key and key in cache:
        search.last_source = "cache"
        return cache[key]["best"], [(c["cfg"], c["ms"]) for c in cache[key]["all"]]
    search.last_source = "search"
    names = sorted(space)
    timed: Dict[tuple, float] = {}
    results: List[Tuple[dict, float]] = []

    def score(cfg: dict) -> float:
        sig = tuple(cfg[n] for n in names)
        if sig not in timed:
            timed[sig] = min(measure(cfg) for _ in range(reps))
            results.append((dict(cfg), timed[sig]))
        return timed[sig]

    if size(space) <= exhaustive_max:
        for values in itertools.product(*(space[n] for n in names)):
            score(dict(zip(names, values)))
        best = min(results, key=lambda r: r[1])[0]
    else:
        best = {n: space[n][0] for n in names}
        best_ms = score(best)
        for _ in range(sweeps):
            changed = False
            for n in names:
                for v in space[n]:
                    if v == best[n]:
                        continue
                    cand = dict(best)
                    cand[n] = v
                    ms = score(cand)
                    if ms < best_ms:
                        best, best_ms, changed = cand, ms, True
            if not changed:
                break
    if key:
        cache = _load()
        cache[key] = {"best": best, "all": [{"cfg": c, "ms": m} for c, m in results], "when": time.time()}
        _store(cache)
    return best, results


search.last_source = "search"
