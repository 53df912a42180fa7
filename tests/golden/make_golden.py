"""Generates the golden fixtures in this folder by running the reference's own
CPU code (oracle/_ref/liboracle_ref.so: UniformGridAccStructBuilder +
UniformGridAccStruct compiled unmodified against the vr shim) on small seeded
scenes.  The reference hard-codes k = 6 cells per triangle
(src/rtplugins/UniformGridAccStructBuilder.cpp:91), so every fixture uses k = 6.

Run from the repository root where the reference checkout exists:
    make -C oracle ref && python tests/golden/make_golden.py
Each .npz holds the inputs (verts, idx, rays, shadow_rays) and the reference's
outputs (grid parameters, CSR offsets / ids, closest hits, occlusion).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "grid-rt_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import pyoracle  # noqa: E402
from gridrt import scenes  # noqa: E402

K = 6


def shadow_rays_from_hits(verts, idx, rays, hits, light):
    """Shadow rays toward a point light from each hit (flat normal turned to
    face the ray, origin offset 2e-4, unnormalised direction, tmax = 1) --
    the setup of SimplePointLight::illuminate / Sample::initShadowRay."""
    ok = hits["id"] >= 0
    r = rays[ok]
    tid = hits["id"][ok]
    v0 = verts[idx[tid, 0]].astype(np.float64)
    e1 = verts[idx[tid, 1]].astype(np.float64) - v0
    e2 = verts[idx[tid, 2]].astype(np.float64) - v0
    n = np.cross(e1, e2)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    d = r[:, 4:7].astype(np.float64)
    flip = (n * d).sum(1) > 0
    n[flip] = -n[flip]
    p = r[:, 0:3] + d * hits["t"][ok, None] + n * 2e-4
    L = light[None, :].astype(np.float64) - p
    keep = (n * L).sum(1) > 0
    out = np.zeros((int(keep.sum()), 8), np.float32)
    out[:, 0:3] = p[keep]
    out[:, 3] = np.float32(2e-4)
    out[:, 4:7] = L[keep]
    out[:, 7] = 1.0
    return out


def write(name, verts, idx, rays, light=None):
    ref = pyoracle.RefScene(verts, idx)
    off, ids = ref.csr()
    h = ref.trace(rays)
    data = dict(verts=verts, idx=idx, k=np.int32(K), res=np.array(ref.info["res"], np.int32),
                bmin=ref.info["bmin"], bmax=ref.info["bmax"], cell=ref.info["cell"], inv_cell=ref.info["inv_cell"],
                offsets=off, ids=ids, rays=rays, hit_id=h["id"], hit_t=h["t"], hit_u=h["u"], hit_v=h["v"])
    if light is not None:
        sr = shadow_rays_from_hits(verts, idx, rays, h, light)
        hs = ref.trace(sr)
        data["shadow_rays"] = sr
        data["occluded"] = ((hs["id"] >= 0) & (hs["t"] < sr[:, 7])).astype(np.uint8)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **data)
    print(f"{path}: {idx.shape[0]} tris, res {ref.info['res']}, {ref.info['nrefs']} refs, "
          f"{rays.shape[0]} rays, {int((h['id'] >= 0).sum())} hits, {os.path.getsize(path)} bytes")


def main():
    if not pyoracle.ref_available():
        raise SystemExit("oracle/_ref/liboracle_ref.so missing: run `make -C oracle ref` first")
    rng = np.random.default_rng(scenes.SEED_BASE + 100)

    sc = scenes.tiny_scene(scenes.SEED_BASE + 101, 300, spread=1.0, size=0.25)
    write("soup300", sc.verts, sc.idx, scenes.random_rays(rng, 3000, (-1.2,) * 3, (1.2,) * 3))

    sc = scenes.plane_and_debris(seed=scenes.SEED_BASE + 102, quads=16, debris=512)
    cam = scenes.plane_and_debris_camera(48, 48)
    write("plane16_debris512", sc.verts, sc.idx, scenes.camera_rays(cam), light=scenes.PLANE_LIGHT)

    v, idx, nrm = scenes.sphere_mesh(lat=24, lon=48)
    sv = scenes.deform(v, nrm, 3)
    cam = scenes.deforming_sphere_camera(48, 48)
    write("sphere24x48_f3", sv, idx, scenes.camera_rays(cam), light=scenes.SPHERE_LIGHT)

    tri = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]], np.float32)
    rays = scenes.random_rays(rng, 500, (-0.5, -0.5, -0.5), (1.5, 1.5, 0.5))
    write("single_planar", tri, np.array([[0, 1, 2]], np.int32), rays)


if __name__ == "__main__":
    main()
