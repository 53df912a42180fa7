"""Edge cases of the trace entry points against the oracle: no rays,
axis-parallel directions (zero and negative-zero components, infinite
1/dir), rays starting inside the grid or missing it, empty [tnear, tfar]
windows, short tfar, any-hit slots without a ray, a one-triangle scene."""
import numpy as np
import pytest

import parity
from gridrt import scenes

pytestmark = pytest.mark.gpu


def _scene(gridlib, sc, k):
    s = gridlib.Scene(0)
    s.set_geometry(sc.verts, sc.idx)
    s.build(k)
    return s


def _rays(o, d, tnear=2e-4, tfar=np.float32(np.finfo(np.float32).max)):
    o = np.asarray(o, np.float32).reshape(-1, 3)
    d = np.asarray(d, np.float32).reshape(-1, 3)
    r = np.empty((o.shape[0], 8), np.float32)
    r[:, 0:3] = o
    r[:, 3] = tnear
    r[:, 4:7] = d
    r[:, 7] = tfar
    return r


def test_no_rays(gridlib):
    sc = scenes.tiny_scene(1, 100)
    s = _scene(gridlib, sc, 4)
    assert s.trace_nearest(np.zeros((0, 8), np.float32)).shape == (0, 4)
    assert s.trace_any(np.zeros((0, 8), np.float32)).shape == (0,)


def test_axis_parallel_rays(gridlib, oracle):
    """Directions along the axes, with +0 and -0 in the other components:
    1/dir is infinite there and the walk must still agree with the oracle."""
    sc = scenes.plane_and_debris()
    s = _scene(gridlib, sc, 4)
    g = oracle.Grid(sc.verts, sc.idx, 4)
    rng = np.random.default_rng(3)
    n = 4000
    o = rng.uniform((-1.2, -0.2, -1.2), (1.2, 1.2, 1.2), size=(n, 3))
    dirs = []
    for axis in range(3):
        for sign in (1.0, -1.0):
            for zsign in (0.0, -0.0):
                d = np.full(3, zsign)
                d[axis] = sign
                dirs.append(d)
    d = np.array(dirs)[rng.integers(0, len(dirs), size=n)]
    rays = _rays(o, d)
    gh = gridlib.split_hits(s.trace_nearest(rays))
    oh = g.trace_closest(rays)
    st = parity.compare_hits(gh, oh, sc.verts, sc.idx, rays, oracle)
    print("\n[axis-parallel]", {k: v for k, v in st.items() if k not in ("unexplained_examples", "fp64")})
    parity.assert_parity(st)
    assert (oh["id"] >= 0).sum() > 500
    rays[:, 7] = 0.5
    parity.check_occlusion("axis-parallel", s, g, gridlib.split_hits, rays, s.trace_any(rays), g.trace_any(rays),
                           sc.verts, sc.idx, oracle)


def test_windows_inside_outside_and_short(gridlib, oracle):
    sc = scenes.tiny_scene(2, 3000, spread=0.8)
    s = _scene(gridlib, sc, 4)
    g = oracle.Grid(sc.verts, sc.idx, 4)
    rng = np.random.default_rng(9)
    n = 6000
    r = scenes.random_rays(rng, n, (-0.9, -0.9, -0.9), (0.9, 0.9, 0.9))   # start inside the grid
    out = scenes.random_rays(rng, n, (3.0, 3.0, 3.0), (4.0, 4.0, 4.0))    # outside; most miss the box
    empty = r.copy()
    empty[:, 3], empty[:, 7] = 1.0, 0.5                                   # tnear > tfar: nothing
    short = r.copy()
    short[:, 7] = rng.uniform(1e-4, 0.05, size=n).astype(np.float32)      # a short segment
    far = r.copy()
    far[:, 3] = rng.uniform(0.1, 0.5, size=n).astype(np.float32)          # a late start
    rays = np.concatenate([r, out, empty, short, far])
    gh = gridlib.split_hits(s.trace_nearest(rays))
    oh = g.trace_closest(rays)
    st = parity.compare_hits(gh, oh, sc.verts, sc.idx, rays, oracle)
    parity.assert_parity(st)
    assert (gh["id"][2 * n:3 * n] < 0).all()
    occ = s.trace_any(rays)
    parity.check_occlusion("windows", s, g, gridlib.split_hits, rays, occ, g.trace_any(rays), sc.verts, sc.idx,
                           oracle)


def test_any_hit_slots_without_ray(gridlib, oracle):
    sc = scenes.tiny_scene(3, 2000)
    s = _scene(gridlib, sc, 4)
    g = oracle.Grid(sc.verts, sc.idx, 4)
    rng = np.random.default_rng(4)
    rays = scenes.random_rays(rng, 5000, (-1, -1, -1), (1, 1, 1))
    rays[:, 7] = 0.7
    rays[::3, 7] = -1.0
    occ = s.trace_any(rays)
    assert (occ[::3] == 2).all()
    keep = np.ones(rays.shape[0], bool)
    keep[::3] = False
    rk = np.ascontiguousarray(rays[keep])
    parity.check_occlusion("slots", s, g, gridlib.split_hits, rk, occ[keep], g.trace_any(rk), sc.verts, sc.idx, oracle)
    assert set(np.unique(occ[keep])) <= {0, 1}


def test_one_triangle(gridlib, oracle):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    idx = np.array([[0, 1, 2]], np.int32)
    s = gridlib.Scene(0)
    s.set_geometry(v, idx)
    s.build(6)
    g = oracle.Grid(v, idx, 6)
    rng = np.random.default_rng(5)
    o = np.column_stack([rng.uniform(-0.2, 1.2, 2000), rng.uniform(-0.2, 1.2, 2000), np.full(2000, 1.0)])
    rays = _rays(o, np.tile([0.0, 0.0, -1.0], (2000, 1)))
    gh = gridlib.split_hits(s.trace_nearest(rays))
    oh = g.trace_closest(rays)
    inside = (o[:, 0] > 0.01) & (o[:, 1] > 0.01) & (o[:, 0] + o[:, 1] < 0.99)
    assert (gh["id"][inside] == 0).all()
    st = parity.compare_hits(gh, oh, v, idx, rays, oracle)
    parity.assert_parity(st)


def test_tuning_values_checked(gridlib):
    """Every launch-shape setting outside its documented values is refused
    with RTG_INVALID_PARAM and leaves the scene's tuning as it was (a trace
    after the refusals equals one before them)."""
    sc = scenes.tiny_scene(3, 200)
    s = gridlib.Scene(0)
    s.set_geometry(sc.verts, sc.idx)
    s.build(4)
    rays = scenes.random_rays(np.random.default_rng(5), 4096, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0))
    before = s.trace_nearest(rays).view(np.int32).copy()
    lib = gridlib.load()
    bad = [(gridlib.RTG_TUNE_EMPTY_RUN, 3), (gridlib.RTG_TUNE_HEAVY_CELL, -1), (gridlib.RTG_TUNE_HEAVY_LANES, 5),
           (gridlib.RTG_TUNE_REFILL, 33), (gridlib.RTG_TUNE_BLOCK, 100), (gridlib.RTG_TUNE_LANES, 3),
           (gridlib.RTG_TUNE_LANES, 0), (99, 1)]
    for key, value in bad:
        assert lib.rtg_scene_set_tuning(s.h, key, value) == gridlib.RTG_INVALID_PARAM, (key, value)
    assert np.array_equal(before, s.trace_nearest(rays).view(np.int32))
