"""Grid build on the GPU vs the oracle: bit-exact CSR (offsets and sorted ids)
and bit-exact grid parameters (box, resolution, cell size, 1/cell size)."""
import numpy as np
import pytest

from gridrt import scenes

pytestmark = pytest.mark.gpu


def _check_grid(gridlib, oracle, verts, idx, k, scene=None):
    s = scene or gridlib.Scene(0)
    s.set_geometry(verts, idx)
    s.build(k)
    info = s.info()
    g = oracle.Grid(verts, idx, k)
    oi = g.info.as_dict()
    assert info["res"] == oi["res"], (info, oi)
    for key in ("bmin", "bmax", "cell", "inv_cell"):
        assert np.array_equal(info[key].view(np.uint32), oi[key].view(np.uint32)), (key, info[key], oi[key])
    assert info["ncells"] == oi["ncells"] and info["nrefs"] == oi["nrefs"]
    off, ids = s.download()
    assert np.array_equal(off, g.offsets), "offsets differ"
    assert np.array_equal(ids, g.ids), "sorted cell lists differ"
    return s, g


@pytest.mark.parametrize("seed", range(12))
@pytest.mark.parametrize("k", [1, 2, 4, 6, 8])
def test_tiny_soups(gridlib, oracle, seed, k):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 600))
    sc = scenes.tiny_scene(seed, n, spread=float(rng.uniform(0.1, 5.0)), size=float(rng.uniform(0.01, 1.0)))
    _check_grid(gridlib, oracle, sc.verts, sc.idx, k)


@pytest.mark.parametrize("k", [4, 6])
def test_plane_and_debris(gridlib, oracle, k):
    sc = scenes.plane_and_debris()
    _check_grid(gridlib, oracle, sc.verts, sc.idx, k)


@pytest.mark.parametrize("k", [2, 4, 8])
@pytest.mark.parametrize("frame", [0, 7])
def test_deforming_sphere(gridlib, oracle, k, frame):
    sc = scenes.deforming_sphere(frame)
    s, g = _check_grid(gridlib, oracle, sc.verts, sc.idx, k)
    if k == 2:
        # every sort class but the bitmap one: thread (2..8), warp lanes
        # (9..32), warp registers (33..256), block bitonic (257..4096)
        counts = np.diff(g.offsets)
        for lo, hi in ((2, 8), (9, 32), (33, 256), (257, 4096)):
            assert ((counts >= lo) & (counts <= hi)).any(), (lo, hi)


def test_skewed_density(gridlib, oracle):
    sc = scenes.skewed_density()
    s, g = _check_grid(gridlib, oracle, sc.verts, sc.idx, 4)
    counts = np.diff(g.offsets)
    # per-cell sort classes: thread (2..8) and warp lanes (9..32) sharing
    # one queue from both ends, block bitonic (257..4096), block bitmap (>4096)
    for lo, hi in ((2, 8), (9, 32), (257, 4096), (4097, 1 << 30)):
        assert ((counts >= lo) & (counts <= hi)).any(), (lo, hi)


@pytest.mark.parametrize("n,k", [(1 << 18, 4), (1 << 20, 8), (1 << 22, 1)])
def test_crowded_cells_rebuild(gridlib, oracle, n, k):
    """Crowded cells, built and rebuilt in one scene: the same bits every time
    and the oracle's.  1M triangles at k = 8 is the skewed benchmark's grid
    (lists up to 70,153, all ids inside one bitmap span: the block sort reads
    the list directly); 4M triangles at k = 1 has lists of ids spread over
    more than one bitmap span (scratch copy, chunked bitmap passes)."""
    sc = scenes.skewed_density(n=n)
    s, g = _check_grid(gridlib, oracle, sc.verts, sc.idx, k)
    assert np.diff(g.offsets).max() >= 1024
    for _ in range(2):
        s.build(k)
        off, ids = s.download()
        assert np.array_equal(off, g.offsets), "offsets differ"
        assert np.array_equal(ids, g.ids), "sorted cell lists differ"


def test_single_and_planar(gridlib, oracle):
    # one triangle in the z = 0 plane: planar box axis gets the 0.01 tolerance
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    _check_grid(gridlib, oracle, v, np.array([[0, 1, 2]], np.int32), 6)
    # axis-aligned sheet of triangles
    sc = scenes.plane_and_debris(quads=16, debris=0)
    _check_grid(gridlib, oracle, sc.verts, sc.idx, 4)


def test_empty_scene(gridlib):
    s = gridlib.Scene(0)
    s.set_geometry(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32))
    s.build(4)
    info = s.info()
    assert info["built"] and info["ncells"] == 0
    hits = s.trace_nearest(scenes.camera_rays(scenes.plane_and_debris_camera(8, 8)))
    assert (hits[:, 0].view(np.int32) == -1).all()


def test_rebuild_deterministic_and_regrow(gridlib, oracle):
    s = gridlib.Scene(0)
    small = scenes.tiny_scene(3, 50)
    _check_grid(gridlib, oracle, small.verts, small.idx, 4, scene=s)
    big = scenes.plane_and_debris()
    _check_grid(gridlib, oracle, big.verts, big.idx, 4, scene=s)      # buffers grow
    off1, ids1 = s.download()
    s.build(4)
    off2, ids2 = s.download()
    assert np.array_equal(off1, off2) and np.array_equal(ids1, ids2)
    _check_grid(gridlib, oracle, small.verts, small.idx, 4, scene=s)  # and shrink in use


def test_device_deform_then_build(gridlib, oracle):
    import torch
    v, idx, nrm = scenes.sphere_mesh()
    s = gridlib.Scene(0)
    s.set_geometry(v, idx)
    d_base = torch.from_numpy(v).cuda()
    d_nrm = torch.from_numpy(nrm).cuda()
    torch.cuda.synchronize()
    for frame in (0, 3, 11):
        s.deform(d_base, d_nrm, 0.05, 3.0, 0.3 * frame)
        s.build(4)
        # the oracle builds from the device's own deformed vertices
        verts_now = s.download_vertices()
        g = oracle.Grid(verts_now, idx, 4)
        off, ids = s.download()
        assert np.array_equal(off, g.offsets) and np.array_equal(ids, g.ids)
        # the deformation stays within float tolerance of the host formula
        host = scenes.deform(v, nrm, frame)
        assert np.abs(verts_now - host).max() < 1e-5
