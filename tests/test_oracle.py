"""The CPU oracle (C restatement) pinned against the reference's own sources
compiled unmodified (oracle/_ref, present where the reference checkout is)
and against committed golden fixtures produced by that compiled reference."""
import glob
import os

import numpy as np
import pytest

from gridrt import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def _ref(oracle):
    if not oracle.ref_available():
        pytest.skip("compiled reference (oracle/_ref) not present on this machine")
    return oracle


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("seed", range(8))
def test_restatement_equals_reference_soups(oracle, seed):
    _ref(oracle)
    rng = np.random.default_rng(100 + seed)
    sc = scenes.tiny_scene(100 + seed, int(rng.integers(1, 3000)), spread=float(rng.uniform(0.2, 4.0)),
                           size=float(rng.uniform(0.01, 0.8)))
    ref = oracle.RefScene(sc.verts, sc.idx)
    g = oracle.Grid(sc.verts, sc.idx, oracle.RefScene.K)
    gi = g.info.as_dict()
    assert ref.info["res"] == gi["res"]
    for k in ("bmin", "bmax", "cell", "inv_cell"):
        assert np.array_equal(_bits(ref.info[k]), _bits(gi[k])), k
    off, ids = ref.csr()
    assert np.array_equal(off, g.offsets) and np.array_equal(ids, g.ids)
    assert np.array_equal(_bits(ref.triaccel()), _bits(g.acc))
    rays = scenes.random_rays(rng, 4000, (-4, -4, -4), (4, 4, 4))
    hr = ref.trace(rays)
    ho = g.trace_closest(rays)
    for k in ("id", "t", "u", "v"):
        assert np.array_equal(_bits(hr[k]), _bits(ho[k])), k


def test_restatement_equals_reference_plane(oracle):
    _ref(oracle)
    sc = scenes.plane_and_debris()
    ref = oracle.RefScene(sc.verts, sc.idx)
    g = oracle.Grid(sc.verts, sc.idx, 6)
    off, ids = ref.csr()
    assert np.array_equal(off, g.offsets) and np.array_equal(ids, g.ids)
    rays = scenes.camera_rays(scenes.plane_and_debris_camera(256, 256))
    hr, ho = ref.trace(rays), g.trace_closest(rays)
    for k in ("id", "t", "u", "v"):
        assert np.array_equal(_bits(hr[k]), _bits(ho[k])), k


def test_restatement_equals_reference_crowded(oracle):
    """A skewed-density scene (90% of the triangles in a 0.1^3 cluster): a
    cell list of tens of thousands of entries, and rays into the cluster."""
    _ref(oracle)
    sc = scenes.skewed_density(n=1 << 15)
    ref = oracle.RefScene(sc.verts, sc.idx)
    g = oracle.Grid(sc.verts, sc.idx, oracle.RefScene.K)
    off, ids = ref.csr()
    assert np.array_equal(off, g.offsets) and np.array_equal(ids, g.ids)
    assert np.diff(off).max() > 4096      # one cluster cell of 29,491 entries at k = 6
    rng = np.random.default_rng(7)
    rays = np.concatenate([scenes.camera_rays(scenes.skewed_density_camera(96, 96)),
                           scenes.random_rays(rng, 3000, (-0.06,) * 3, (0.06,) * 3)])
    hr, ho = ref.trace(rays), g.trace_closest(rays)
    for k in ("id", "t", "u", "v"):
        assert np.array_equal(_bits(hr[k]), _bits(ho[k])), k


def test_grid_walk_equals_brute_force_mostly(oracle):
    """Sanity of the reference itself: the grid walk returns the brute-force
    closest hit for almost every ray (exceptions are the reference's own
    window/epsilon cases)."""
    _ref(oracle)
    sc = scenes.tiny_scene(5, 400, spread=1.0, size=0.3)
    ref = oracle.RefScene(sc.verts, sc.idx)
    rays = scenes.random_rays(np.random.default_rng(1), 3000, (-1, -1, -1), (1, 1, 1))
    a, b = ref.trace(rays), ref.trace(rays, brute=True)
    assert (a["id"] == b["id"]).mean() > 0.99


@pytest.mark.skipif(not GOLDEN, reason="no golden fixtures")
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_matches_golden(oracle, path):
    z = np.load(path)
    verts, idx, k = z["verts"], z["idx"], int(z["k"])
    g = oracle.Grid(verts, idx, k)
    assert tuple(g.info.res) == tuple(z["res"])
    assert np.array_equal(_bits(np.array(g.info.bmin, np.float32)), _bits(z["bmin"]))
    assert np.array_equal(_bits(np.array(g.info.inv_cell, np.float32)), _bits(z["inv_cell"]))
    assert np.array_equal(g.offsets, z["offsets"]) and np.array_equal(g.ids, z["ids"])
    h = g.trace_closest(z["rays"])
    for key in ("id", "t", "u", "v"):
        assert np.array_equal(_bits(h[key]), _bits(z["hit_" + key])), key
    if "shadow_rays" in z:
        assert np.array_equal(g.trace_any(z["shadow_rays"]), z["occluded"])


def test_any_hit_definition(oracle):
    """occluded == closest hit exists with t < tmax (the reference's CPU any-hit
    entry points are stubs, src/rtcore/IAccStruct.cpp:108-122)."""
    sc = scenes.tiny_scene(9, 300, spread=1.0, size=0.3)
    g = oracle.Grid(sc.verts, sc.idx, 4)
    rays = scenes.random_rays(np.random.default_rng(3), 2000, (-1, -1, -1), (1, 1, 1))
    rays[:, 7] = 0.5
    occ = g.trace_any(rays)
    h = g.trace_closest(rays)
    assert np.array_equal(occ, ((h["id"] >= 0) & (h["t"] < 0.5)).astype(np.uint8))


def test_camera_rays_match_reference_formula():
    cam = scenes.plane_and_debris_camera(16, 8)
    rays = scenes.camera_rays(cam)
    # pixel (3, 5): dir = (baseDir + nearU*u) + nearV*v in float32
    i = 5 * 16 + 3
    u = (np.float32(3) + np.float32(0.5)) * (np.float32(1) / np.float32(16))
    v = (np.float32(5) + np.float32(0.5)) * (np.float32(1) / np.float32(8))
    d = (cam.base_dir + cam.near_u * u) + cam.near_v * v
    assert np.array_equal(rays[i, 4:7], d.astype(np.float32))
    assert rays[i, 3] == np.float32(2e-4)
    px, py = scenes.camera_pixel_of_ray(np.arange(64), 8, 8, "morton8")
    assert sorted(zip(px.tolist(), py.tolist())) == [(x, y) for x in range(8) for y in range(8)]
