"""The autotuner's search strategies on a synthetic cost (no GPU): the
exhaustive search over a small space and the coordinate descent over a large
one both find the optimum of a separable cost, the descent timing far fewer
candidates; a cached result is reported as coming from the cache."""
import json

from gridrt import autotune


def _cost(cfg):
    # separable: each dimension has one best value
    return (abs(cfg["empty_run"] - 8) + (0 if cfg["order"] == "scanline" else 3) + abs(cfg["block"] - 64) / 64
            + (0 if cfg["persistent"] else 1) + abs(cfg["heavy_cell"] - 24) / 8 + (cfg["heavy_lanes"] != 16)
            + (not cfg["cell_records"]) + cfg["refill"] / 16 + abs(cfg["lanes"] - 2))


BEST = {"empty_run": 8, "order": "scanline", "block": 64, "persistent": True, "heavy_cell": 24,
        "heavy_lanes": 16, "cell_records": True, "refill": 0, "lanes": 2}


def test_descent_finds_separable_optimum():
    calls = []

    def measure(cfg):
        calls.append(cfg)
        return _cost(cfg)

    best, table = autotune.search(measure, reps=1)
    assert autotune.size(autotune.SPACE) > 256           # the default space takes the descent
    assert best == BEST
    assert len(table) == len(calls) < autotune.size(autotune.SPACE) // 10
    assert autotune.search.last_source == "search"


def test_exhaustive_small_space():
    space = {"order": ("morton8", "scanline"), "empty_run": (2, 4, 8), "block": (128, 64)}

    def measure(cfg):
        return _cost(dict(BEST, **cfg))

    best, table = autotune.search(measure, space=space, reps=2)
    assert len(table) == 12
    assert best == {"order": "scanline", "empty_run": 8, "block": 64}


def test_cache_reports_its_source(tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "cache.json"))
    space = {"empty_run": (2, 4, 8)}
    best, _ = autotune.search(lambda c: abs(c["empty_run"] - 4), space=space, key="w", reps=1)
    assert best == {"empty_run": 4} and autotune.search.last_source == "search"
    best2, _ = autotune.search(lambda c: 0.0, space=space, key="w", reps=1)
    assert best2 == best and autotune.search.last_source == "cache"
    assert "w" in json.load(open(tmp_path / "cache.json"))
