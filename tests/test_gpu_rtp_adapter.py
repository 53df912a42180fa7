"""The C++ plugin mirror (include/gridrt_rtp.hpp): a Geometry built through
UniformGridAccStructBuilder::buildGeometry and traced ray by ray through the
virtual IAccStruct calls gives exactly the batched results, and those match
the oracle under the near-tie rules."""
import json
import os
import subprocess

import numpy as np
import pytest

import parity
from gridrt import build, scenes

pytestmark = pytest.mark.gpu


def test_cpp_plugin_mirror(gridlib, oracle, tmp_path):
    tool = build.tool_path("rtp_adapter_check")
    if not os.path.exists(tool):
        build.build_tools()
    sc = scenes.plane_and_debris(quads=24, debris=3000)
    rng = np.random.default_rng(11)
    rays = np.concatenate([scenes.camera_rays(scenes.plane_and_debris_camera(48, 48)),
                           scenes.random_rays(rng, 1500, (-1, 0, -1), (1, 1, 1))])
    anyr = rays.copy()
    p = str(tmp_path / "case")
    sc.verts.astype(np.float32).tofile(p + ".verts")
    sc.idx.astype(np.int32).tofile(p + ".tris")
    rays.astype(np.float32).tofile(p + ".rays")
    # a frame, rendered once and then as a stream of frames with overlapped read-back
    cam = gridlib.camera_struct(scenes.plane_and_debris_camera(64, 48), "morton8")
    with open(p + ".cam", "wb") as f:
        f.write(bytes(cam) + np.asarray(scenes.PLANE_LIGHT, np.float32).tobytes())
    r = subprocess.run([tool, p + ".verts", p + ".tris", p + ".rays", p, p + ".cam"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert json.loads(r.stdout.strip().splitlines()[-1])["frame_diff"] == 0
    single = np.fromfile(p + ".single.f32", np.float32).reshape(-1, 4)
    batch = np.fromfile(p + ".batch.f32", np.float32).reshape(-1, 4)
    assert np.array_equal(single.view(np.uint32), batch.view(np.uint32))
    # InstancedScene with one identity instance: the same words
    inst = np.fromfile(p + ".inst.f32", np.float32).reshape(-1, 4)
    assert np.array_equal(inst.view(np.uint32), batch.view(np.uint32))
    any_s = np.fromfile(p + ".any_single.u8", np.uint8)
    any_b = np.fromfile(p + ".any_batch.u8", np.uint8)
    assert np.array_equal(any_s, any_b)
    g = oracle.Grid(sc.verts, sc.idx, 4)
    gh = gridlib.split_hits(batch)
    oh = g.trace_closest(rays)
    st = parity.compare_hits(gh, oh, sc.verts, sc.idx, rays, oracle)
    parity.assert_parity(st)
    s = gridlib.Scene(0)
    s.set_geometry(sc.verts, sc.idx)
    s.build(4)
    parity.check_occlusion("adapter", s, g, gridlib.split_hits, anyr, any_b, g.trace_any(anyr), sc.verts, sc.idx,
                           oracle)
