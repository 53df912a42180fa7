"""Loaded meshes build the oracle's grid; double-buffered keyframe staging
gives the same grids and hits as direct vertex updates."""
import numpy as np
import pytest

from gridrt import scenes

pytestmark = pytest.mark.gpu


def test_loaded_obj_builds_oracle_grid(gridlib, oracle, tmp_path):
    sc = scenes.deforming_sphere(4)
    p = tmp_path / "sphere.obj"
    with open(p, "w") as f:
        for v in sc.verts:
            f.write(f"v {float(v[0])!r} {float(v[1])!r} {float(v[2])!r}\n")
        for t in sc.idx:
            f.write(f"f {t[0] + 1} {t[1] + 1} {t[2] + 1}\n")
    verts, tris, src, info = gridlib.load_mesh(p)
    assert info["dropped"] == 0 and tris.shape[0] == sc.ntris and np.array_equal(src, np.arange(sc.ntris))
    s = gridlib.Scene(0)
    got = s.load(p)
    assert got["ntris"] == sc.ntris and got["nverts"] == 3 * sc.ntris
    s.build(4)
    off, ids = s.download()
    g = oracle.Grid(verts, tris, 4)
    assert np.array_equal(off, g.offsets) and np.array_equal(ids, g.ids)
    # same triangles as the indexed input: the same grid
    g2 = oracle.Grid(sc.verts, sc.idx, 4)
    assert np.array_equal(g.offsets, g2.offsets) and np.array_equal(g.ids, g2.ids)


def test_staged_keyframes_equal_direct_updates(gridlib):
    import torch
    v, idx, nrm = scenes.sphere_mesh()
    frames = [torch.from_numpy(scenes.deform(v, nrm, f)).pin_memory() for f in range(6)]
    cam = scenes.deforming_sphere_camera(256, 256)
    n = cam.width * cam.height
    a, b = gridlib.Scene(0), gridlib.Scene(0)
    for s in (a, b):
        s.set_geometry(frames[0].numpy(), idx)
        s.build(4)
    copy = torch.cuda.Stream()
    ha = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    hb = torch.empty_like(ha)
    a.stage_vertices(frames[1], v.shape[0], copy.cuda_stream)
    for f in range(1, 6):
        a.build_async(4)
        if f + 1 < 6:
            a.stage_vertices(frames[f + 1], v.shape[0], copy.cuda_stream)   # overlaps frame f's trace
        a.trace_camera_device(cam, ha, order="morton8")
        b.update_vertices(frames[f], v.shape[0], from_device=False)
        b.build(4)
        b.trace_camera_device(cam, hb, order="morton8")
        torch.cuda.synchronize()
        assert a.build_check() == 0
        assert torch.equal(ha, hb), f
        oa, ia = a.download()
        ob, ib = b.download()
        assert np.array_equal(oa, ob) and np.array_equal(ia, ib), f
