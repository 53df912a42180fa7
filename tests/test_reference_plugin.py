"""The reference-side binding (include/gridrt_reference_plugin.hpp) compiled
against the reference's own headers (rt/IAccStructBuilder.h, rt/IAccStruct.h,
rt/Geometry.h, with this project's vr shim) and linked with libgridrt.so and
the reference's own CPU plugin (compiled from its sources into oracle/_ref).

tests/cpp/reference_plugin_check.cpp builds one rt::Geometry with the
reference's rtp::UniformGridAccStructBuilder and one with
rtp::GpuUniformGridAccStructBuilder, through the rt::IAccStructBuilder
interface, and traces the same rays through rt::IAccStruct on both, prepared
as IAccStruct::traceNearestInstance prepares them.  Without a GPU (this test
is not marked gpu) the GPU plugin must fail the reference's way -- silently,
the geometry still owning a structure that reports no hit and leaves the hit
record untouched -- while the CPU plugin traces; where a GPU is present the
hits of the two plugins are compared under the near-tie rules.  Needs the
reference checkout (GRIDRT_REFERENCE_DIR or the oracle recipe's default) and
skips where it is absent (the GPU host has none)."""
import json
import os
import subprocess

import numpy as np
import pytest

import parity
from gridrt import build, scenes

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_include(oracle):
    ref = oracle.reference_dir()
    inc = os.path.join(ref, "include") if ref else ""
    if not inc or not os.path.isfile(os.path.join(inc, "rt", "IAccStructBuilder.h")):
        pytest.skip("reference checkout not present on this machine")
    if not oracle.ref_available():
        pytest.skip("compiled reference (oracle/_ref) not present on this machine")
    return inc


def _build_driver(inc, out):
    lib_dir = os.path.dirname(build.LIB)
    ref_dir = os.path.join(REPO, "oracle", "_ref")
    nv = build.nvcc()
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nv))), "lib64") \
        if os.path.isabs(nv) else "/usr/local/cuda/lib64"
    cmd = ["g++", "-std=c++14", "-O2", "-ffp-contract=off", "-w", "-fopenmp", "-include", "cstring",
           "-include", "cstdio", "-I", os.path.join(REPO, "oracle", "shim"), "-I", inc,
           "-I", os.path.join(REPO, "include"), os.path.join(REPO, "tests", "cpp", "reference_plugin_check.cpp"),
           "-o", out, "-L", lib_dir, "-lgridrt", f"-Wl,-rpath,{lib_dir}", "-L", ref_dir, "-l:liboracle_ref.so",
           f"-Wl,-rpath,{ref_dir}", "-L", cuda_lib, "-lcudart", f"-Wl,-rpath,{cuda_lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, " ".join(cmd) + "\n" + r.stderr


def test_reference_side_binding_against_reference_headers(gridlib, oracle, tmp_path):
    inc = _reference_include(oracle)
    gridlib.load()
    tool = str(tmp_path / "reference_plugin_check")
    _build_driver(inc, tool)
    sc = scenes.plane_and_debris(quads=24, debris=3000)
    rng = np.random.default_rng(13)
    rays = np.concatenate([scenes.camera_rays(scenes.plane_and_debris_camera(48, 48)),
                           scenes.random_rays(rng, 1500, (-1, 0, -1), (1, 1, 1))])
    p = str(tmp_path / "case")
    sc.verts.astype(np.float32).tofile(p + ".verts")
    sc.idx.astype(np.int32).tofile(p + ".tris")
    rays.astype(np.float32).tofile(p + ".rays")
    r = subprocess.run([tool, p + ".verts", p + ".tris", p + ".rays", "6", p], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    print("\n[reference plugin]", out)
    n = rays.shape[0]
    assert out["rays"] == n and out["gpu_has_struct"]
    # the reference's own plugin traced the rays: its hits are the oracle's
    cpu = gridlib.split_hits(np.fromfile(p + ".cpu.f32", np.float32).reshape(-1, 4))
    ref = oracle.Grid(sc.verts, sc.idx, 6).trace_closest(rays)
    assert out["cpu_hits"] > n // 10
    assert np.array_equal(cpu["id"], ref["id"])
    if not out["gpu_ok"]:
        # no GPU: the build failed without throwing, every trace left the hit alone
        assert out["gpu_status"] != 0 and out["gpu_hits"] == 0 and out["gpu_untouched"] == n
        return
    gpu = gridlib.split_hits(np.fromfile(p + ".gpu.f32", np.float32).reshape(-1, 4))
    st = parity.compare_hits(gpu, cpu, sc.verts, sc.idx, rays, oracle)
    parity.assert_parity(st)
    assert out["instance_ok"] == out["gpu_hits"]
