"""rtg_grid_build_noalloc: the grid build that allocates no device memory.

It is for callers that must not let the library allocate GPU memory (frame
loops that cannot absorb an allocation's latency, applications that hand out
all device memory from their own pool).  The test gives it buffers allocated
here, calls it twice in a row through the C ABI on two different scenes, and
checks each result against the regular entry point (rtg_scene_build +
rtg_scene_grid_download): offsets and sorted ids are integers and must match
exactly; the triangle records must equal v0|id, v1 - v0, v2 - v0 in float32.
It runs last (file name) so a failure here cannot hide the other tests.
"""
import ctypes

import numpy as np
import pytest

from gridrt import scenes

pytestmark = pytest.mark.gpu


def _noalloc_build(lib, L, verts, idx, k):
    import torch
    d_verts = torch.from_numpy(np.ascontiguousarray(verts, np.float32)).cuda()
    d_tris = torch.from_numpy(np.ascontiguousarray(idx, np.int32)).cuda()
    info = lib.GridInfo()
    # outputs sized generously: cells ~ k * triangles (plus box-surface terms),
    # references up to the entry point's own limit
    off = torch.full((4 * k * idx.shape[0] + 1024,), -7, dtype=torch.int32, device="cuda")
    ids = torch.full((1 << 19,), -7, dtype=torch.int32, device="cuda")
    rec = torch.empty((idx.shape[0], 12), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = L.rtg_grid_build_noalloc(d_verts.data_ptr(), verts.shape[0], d_tris.data_ptr(), idx.shape[0], k,
                                  off.data_ptr(), off.numel(), ids.data_ptr(), ids.numel(), rec.data_ptr(),
                                  ctypes.byref(info), None)
    assert rc == lib.RTG_OK, (rc, L.rtg_last_error())
    torch.cuda.synchronize()
    n_c, n_r = info.ncells + 1, info.nrefs
    return info.as_dict(), off[:n_c].cpu().numpy(), ids[:n_r].cpu().numpy(), rec.cpu().numpy()


def _regular_build(lib, verts, idx, k):
    s = lib.Scene(0)
    s.set_geometry(verts, idx)
    s.build(k)
    info = s.info()
    off, ids = s.download()
    s.close()
    return info, off, ids


def _expected_records(verts, idx):
    v0 = verts[idx[:, 0]]
    rec = np.zeros((idx.shape[0], 12), np.float32)
    rec[:, 0:3] = v0
    rec[:, 3] = np.arange(idx.shape[0], dtype=np.int32).view(np.float32)
    rec[:, 4:7] = verts[idx[:, 1]] - v0
    rec[:, 8:11] = verts[idx[:, 2]] - v0
    return rec


def test_noalloc_matches_regular_build_twice(gridlib):
    L = gridlib.load()
    cases = [(scenes.plane_and_debris(), 4), (scenes.deforming_sphere(7), 2)]
    for sc, k in cases:     # two calls in a row; the second must not see the first's state
        info_a, off_a, ids_a, rec = _noalloc_build(gridlib, L, sc.verts, sc.idx, k)
        info_b, off_b, ids_b = _regular_build(gridlib, sc.verts, sc.idx, k)
        assert info_a["res"] == info_b["res"] and info_a["nrefs"] == info_b["nrefs"]
        for key in ("bmin", "bmax", "cell", "inv_cell"):
            assert np.array_equal(info_a[key].view(np.uint32), info_b[key].view(np.uint32)), key
        assert np.array_equal(off_a, off_b), "offsets differ from rtg_scene_build"
        assert np.array_equal(ids_a, ids_b), "sorted cell lists differ from rtg_scene_build"
        assert np.array_equal(rec.view(np.uint32), _expected_records(sc.verts, sc.idx).view(np.uint32))


def test_noalloc_reports_sizes_when_buffers_are_small(gridlib):
    import torch
    L = gridlib.load()
    sc = scenes.plane_and_debris(quads=32, debris=1024)
    d_verts = torch.from_numpy(sc.verts).cuda()
    d_tris = torch.from_numpy(sc.idx).cuda()
    rec = torch.empty((sc.ntris, 12), dtype=torch.float32, device="cuda")
    small = torch.empty(4, dtype=torch.int32, device="cuda")
    info = gridlib.GridInfo()
    torch.cuda.synchronize()
    rc = L.rtg_grid_build_noalloc(d_verts.data_ptr(), sc.nverts, d_tris.data_ptr(), sc.ntris, 4, small.data_ptr(),
                                  small.numel(), small.data_ptr(), small.numel(), rec.data_ptr(), ctypes.byref(info),
                                  None)
    assert rc == gridlib.RTG_NO_MEMORY and info.ncells > 3       # offsets too small: cell count reported
    off = torch.empty(info.ncells + 1, dtype=torch.int32, device="cuda")
    rc = L.rtg_grid_build_noalloc(d_verts.data_ptr(), sc.nverts, d_tris.data_ptr(), sc.ntris, 4, off.data_ptr(),
                                  off.numel(), small.data_ptr(), small.numel(), rec.data_ptr(), ctypes.byref(info),
                                  None)
    assert rc == gridlib.RTG_NO_MEMORY and info.nrefs > 4         # ids too small: reference count reported


def test_noalloc_rejects_grids_over_its_limit(gridlib):
    import torch
    L = gridlib.load()
    sc = scenes.skewed_density(n=1 << 18)        # far more than 524,288 references
    d_verts = torch.from_numpy(sc.verts).cuda()
    d_tris = torch.from_numpy(sc.idx).cuda()
    off = torch.empty(1 << 22, dtype=torch.int32, device="cuda")
    ids = torch.empty(1 << 22, dtype=torch.int32, device="cuda")
    rec = torch.empty((sc.ntris, 12), dtype=torch.float32, device="cuda")
    info = gridlib.GridInfo()
    torch.cuda.synchronize()
    rc = L.rtg_grid_build_noalloc(d_verts.data_ptr(), sc.nverts, d_tris.data_ptr(), sc.ntris, 4, off.data_ptr(),
                                  off.numel(), ids.data_ptr(), ids.numel(), rec.data_ptr(), ctypes.byref(info), None)
    assert rc == gridlib.RTG_INVALID_PARAM and info.nrefs > (1 << 19)
    # the shared working array is usable straight after the rejected call
    good = scenes.plane_and_debris(quads=48, debris=4096)
    _check_against_regular(gridlib, L, good.verts, good.idx, 4)


def _check_against_regular(gridlib, L, verts, idx, k):
    info_a, off_a, ids_a, rec = _noalloc_build(gridlib, L, verts, idx, k)
    info_b, off_b, ids_b = _regular_build(gridlib, verts, idx, k)
    assert info_a["res"] == info_b["res"] and info_a["nrefs"] == info_b["nrefs"]
    for key in ("bmin", "bmax", "cell", "inv_cell"):
        assert np.array_equal(info_a[key].view(np.uint32), info_b[key].view(np.uint32)), key
    assert np.array_equal(off_a, off_b), "offsets differ from rtg_scene_build"
    assert np.array_equal(ids_a, ids_b), "sorted cell lists differ from rtg_scene_build"
    assert np.array_equal(rec.view(np.uint32), _expected_records(verts, idx).view(np.uint32))
    return info_a, off_a, ids_a


def _resolution_is_ambiguous(verts, ntris, k):
    """Whether the resolution rule sits on a powf ulp boundary, in float32:
    the grid box enlarged by 1% (Aabb::scaleBy), V, k * N / V, f = pow(q, 1/3)
    rounded from double, and whether ceil(extent * f) changes between
    f - 1 ulp and f + 1 ulp on some axis.  The device flags a build whenever
    ceil changes across a wider band around its own powf (then the host's
    powf decides the resolution), so such a scene always takes that path."""
    f32 = np.float32
    mn, mx = verts.min(0).astype(f32), verts.max(0).astype(f32)
    s = np.where(mn == mx, f32(0.01), (np.abs(mx - mn) * f32(0.01)).astype(f32)).astype(f32)
    mn, mx = (mn - s).astype(f32), (mx + s).astype(f32)
    d = (mx - mn).astype(f32)
    V = f32(f32(d[0] * d[1]) * d[2])
    q = f32(f32(k * ntris) / V)
    f = f32(np.float64(q) ** np.float64(f32(1.0) / f32(3.0)))
    fm, fp = np.nextafter(f, f32(0.0)), np.nextafter(f, f32(np.inf))
    return bool((np.ceil((d * fm).astype(f32)) != np.ceil((d * fp).astype(f32))).any())


def _ambiguous_scene(k=4, n=200, seed=5):
    """A soup of n small triangles in the unit cube plus one triangle
    (0,0,0), (0.5,1,1), (X,0.5,0.5) whose x extent X is chosen, by search over
    float32 values, so that the resolution rule sits on a powf ulp boundary."""
    rng = np.random.default_rng(seed)
    cent = rng.uniform(0.05, 0.95, size=(n, 3)).astype(np.float32)
    soup = (cent[:, None, :] + rng.uniform(-0.03, 0.03, size=(n, 3, 3))).astype(np.float32).reshape(-1, 3)
    for i in range(2_000_000):
        X = np.float32(1.0 + 1e-6 * i)
        verts = np.concatenate([soup, np.array([[0, 0, 0], [0.5, 1, 1], [X, 0.5, 0.5]], np.float32)])
        if _resolution_is_ambiguous(verts, n + 1, k):
            idx = np.arange(3 * (n + 1), dtype=np.int32).reshape(-1, 3)
            return verts, idx
    raise AssertionError("no ambiguous extent found")


def test_noalloc_host_resolved_parameters(gridlib, oracle):
    """A scene whose resolution depends on the last ulp of powf takes the
    path where the call re-resolves the parameters on the host and clears
    the sort counters in the shared array by hand: the grid still equals
    rtg_scene_build's and the oracle's, also on a second call in a row."""
    L = gridlib.load()
    verts, idx = _ambiguous_scene()
    for _ in range(2):
        info, off, ids = _check_against_regular(gridlib, L, verts, idx, 4)
        g = oracle.Grid(verts, idx, 4)
        assert np.array_equal(off, g.offsets) and np.array_equal(ids, g.ids)
    # and an ordinary build right after it
    sc = scenes.plane_and_debris(quads=40, debris=3000)
    _check_against_regular(gridlib, L, sc.verts, sc.idx, 4)
