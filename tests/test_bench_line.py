"""The bench's one result line (no GPU): built from a full result of the
default run on a GB300 (tests/fixtures/bench_detail_gb300.json, written by
`bench.py --detail`), it carries every key of the result-line contract, the
roofline, CPU-baseline, end-to-end, launch-count and clock objects, one
small object per further workload, and stays a few KB long.  The reference
arm's line, run here on the host cores, names the same metric and workload."""
import importlib.util
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def _bench():
    spec = importlib.util.spec_from_file_location("bench", os.path.join(HERE, "..", "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_default_line_contract():
    bench = _bench()
    with open(os.path.join(HERE, "fixtures", "bench_detail_gb300.json")) as f:
        d = json.load(f)
    subs = {"cfg0_plain": d["cfg0_plain"], "cfg2_skewed": bench.compact_skewed(d["cfg2_skewed"]),
            "cfg3_batched": bench.compact_batched(d["cfg3_batched"]),
            "cfg4_serving": bench.compact_serving(d["cfg4_serving"])}
    line = bench.compact_line(d["deforming"], subs)
    text = json.dumps(line, separators=(",", ":"))
    assert len(text) < 4096, len(text)
    back = json.loads(text)
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e",
                "gpu_launches", "clocks"):
        assert key in back, key
    assert back["value"] > 0 and back["n_gpus"] == 1 and back["higher_is_better"] is True
    assert back["warmup"] >= 3 and back["scaling"] == "weak"
    assert back["config"]["workload"] and "l2" in back["config"]
    rf = back["roofline"]
    assert rf["bound"] in ("hbm", "tensor") and 0 < rf["frac"] < 2 and rf["achieved"] > 0 and rf["peak"] > 0
    assert abs(rf["frac"] - rf["achieved"] / rf["peak"]) < 1e-3
    cb = back["cpu_baseline"]
    assert cb["value"] > 0 and cb["cores"] >= 1 and cb["kind"] in ("port", "reference")
    e = back["e2e"]
    assert e["value"] > 0 and e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    assert isinstance(back["gpu_launches"], int) and back["gpu_launches"] > 0
    assert back["clocks"]["sm_mhz"] > 0 and isinstance(back["clocks"]["reasons"], list)
    for name in subs:
        assert name in back and back[name].get("value", 0) > 0, name
    # two frames in flight: the line also carries the one-frame figure
    full = dict(d["deforming"], one_frame_in_flight={"value": 3478.3, "ms_per_step": 0.3792})
    full["config"] = dict(full["config"], frames_in_flight=2)
    two = bench.compact_line(full, subs)
    assert two["config"]["frames_in_flight"] == 2 and "pair" in two["config"]["l2"]
    assert two["one_frame_in_flight"]["value"] == 3478.3
    assert len(json.dumps(two, separators=(",", ":"))) < 4096


def test_reference_arm_line(oracle):
    """`bench.py --impl reference` (the reference's CPU path: single-thread
    grid build and every primary and shadow ray on all host threads) prints
    one line with the GPU arm's metric, unit and workload, its CPU baseline
    and an end-to-end object with no device copies."""
    import subprocess
    import sys
    r = subprocess.run([sys.executable, os.path.join(HERE, "..", "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=os.path.join(HERE, ".."))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, r.stdout
    ref = json.loads(lines[0])
    with open(os.path.join(HERE, "fixtures", "bench_detail_gb300.json")) as f:
        gpu = json.load(f)["deforming"]
    assert ref["impl"] == "reference"
    for key in ("metric", "unit", "higher_is_better", "scaling"):
        assert ref[key] == gpu[key], key
    assert ref["config"]["workload"] == gpu["config"]["workload"] and ref["config"]["k"] == gpu["config"]["k"]
    assert ref["value"] > 0 and ref["steps"] == 1 and ref["warmup"] >= 3
    cb = ref["cpu_baseline"]
    assert cb["value"] == ref["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e = ref["e2e"]
    assert e["value"] == ref["value"] and e["unit"] == ref["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_tuning_text_round_trip():
    """--fixed-tuning text parses into every launch-shape setting (unnamed
    ones at the library's defaults), and the line's short form names each."""
    bench = _bench()
    text = ("k=4,order=morton8,empty_run=4,persistent=1,heavy_cell=32,heavy_lanes=16,cell_records=1,refill=16,"
            "block=256,lanes=2")
    cfg = bench._parse_tuning(text)
    assert cfg == {"k": 4, "order": "morton8", "empty_run": 4, "persistent": True, "heavy_cell": 32,
                   "heavy_lanes": 16, "cell_records": True, "refill": 16, "block": 256, "lanes": 2}
    assert bench._tune_str(cfg) == "morton8/er4/p1/h32x16/r16/c1/b256/l2"
    short = bench._parse_tuning("k=2,order=scanline")
    assert short["persistent"] is False and short["cell_records"] is False
    assert (short["block"], short["lanes"], short["heavy_lanes"], short["refill"]) == (128, 1, 32, 0)
    assert bench._parse_tuning("") is None and bench._tune_str(None) == ""


def test_cpu_tile_order():
    """The CPU arms trace rays in 16 x 16 pixel tiles, row of tiles after row
    of tiles (the reference TiledRenderer's schedule): a permutation of the
    scanline indices whose every run of 256 is one tile."""
    import numpy as np
    bench = _bench()
    w, h = 64, 32
    order = bench._tile_order(w, h)
    assert np.array_equal(np.sort(order), np.arange(w * h))
    for t in range(w * h // 256):
        run = order[256 * t:256 * (t + 1)]
        x, y = run % w, run // w
        assert x.max() - x.min() == 15 and y.max() - y.min() == 15
        assert (x.min(), y.min()) == ((t % (w // 16)) * 16, (t // (w // 16)) * 16)
