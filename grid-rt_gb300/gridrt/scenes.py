"""Seeded synthetic scenes, cameras and rays for the uniform-grid workloads.

The reference's benchmark scenes (the paper's animated models) are not
available; these generators stand in for them with the shapes, sizes and
value distributions of the named workloads:

* ``plane_and_debris``  65,536 triangles: a 128x128-quad ground plane at y=0
  over [-1,1]^2 (32,768 tris, 16,641 shared vertices) plus 32,768 random
  triangles with centroid U([-1,1]x[0,1]x[-1,1]) and vertices offset by
  U[-0.02,0.02]^3.  Pinhole camera eye (0,1.5,3) -> (0,0.3,0), 60 deg, 512^2,
  one ray per pixel centre; point light (2,4,2).
* ``deforming_sphere``  160 latitude bands x 320 longitude segments x 2 =
  102,400 triangles on a unit UV sphere whose two pole caps are left open (the
  ring latitudes are pi*(i+1)/162, i = 0..160) so every triangle has area;
  frame f displaces each vertex by 0.05*sin(3*p.x + 0.3*f) along its radial
  normal.
* ``skewed_density``  1,048,576 triangles: 90% small (edge <= 0.002) in a
  0.1^3 box at the origin, 10% large (edge <= 0.5) in [-4,4]^3.

All arithmetic that decides ray bits is float32 with one rounding per
operation, in the same order as the device ray generator, so host and device
rays are bit-identical.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

SEED_BASE = 20261203

# Rays are 8 float32 words: {ox, oy, oz, tnear, dx, dy, dz, tfar}.
RAY_WORDS = 8
RAY_EPSILON = np.float32(2e-4)      # Context::setRayEpsilon default, src/rtcore/Context.cpp:505
FLT_MAX = np.float32(np.finfo(np.float32).max)


@dataclasses.dataclass
class Scene:
    verts: np.ndarray     # (V, 3) float32
    idx: np.ndarray       # (N, 3) int32
    name: str = ""

    @property
    def ntris(self) -> int:
        return int(self.idx.shape[0])

    @property
    def nverts(self) -> int:
        return int(self.verts.shape[0])


@dataclasses.dataclass
class Camera:
    """Pinhole camera basis as PinholeCamera::newFrame computes it
    (src/rtplugins/PinholeCamera.cpp:23-55): dir = baseDir + nearU*(x/w) +
    nearV*(y/h), unnormalised, row 0 at the bottom."""
    eye: np.ndarray       # (3,) float32
    base_dir: np.ndarray  # (3,) float32
    near_u: np.ndarray    # (3,) float32
    near_v: np.ndarray    # (3,) float32
    width: int
    height: int

    def packed(self) -> np.ndarray:
        """12 float32: eye, baseDir, nearU, nearV (cudaSetCameraParameters order,
        src/rtcuda/RayTracing.h:20-23)."""
        return np.concatenate([self.eye, self.base_dir, self.near_u, self.near_v]).astype(np.float32)


def look_at_camera(eye, center, up, fovy_deg: float, width: int, height: int, znear: float = 1.0) -> Camera:
    """Camera basis from a look-at.  The reference builds the orientation with
    vr::mat4f::makeLookAt (not shipped); this uses the OpenGL look-at basis:
    axisX = normalize(f x up), axisY = axisX x f, axisZ = -f (the camera looks
    down -axisZ, PinholeCamera.cpp:45).  Computed in float64 and rounded once."""
    eye = np.asarray(eye, np.float64)
    f = np.asarray(center, np.float64) - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, np.asarray(up, np.float64))
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    ax, ay, az = s, u, -f
    sz = znear
    sy = sz * math.tan(math.radians(fovy_deg * 0.5))
    sx = sy * width / height
    near_origin = eye + ax * -sx + ay * -sy + az * -sz
    return Camera(eye=eye.astype(np.float32),
                  base_dir=(near_origin - eye).astype(np.float32),
                  near_u=(ax * (2.0 * sx)).astype(np.float32),
                  near_v=(ay * (2.0 * sy)).astype(np.float32),
                  width=int(width), height=int(height))


def camera_pixel_of_ray(ray_index: np.ndarray, width: int, height: int, order: str = "scanline"):
    """Pixel (x, y) of ray i.  'scanline': i = y*w + x.  'morton8': 8x8 tiles in
    scanline order of tiles, Morton (Z) order inside a tile (w, h multiples of 8)."""
    i = np.asarray(ray_index, np.int64)
    if order == "scanline":
        return i % width, i // width
    if order == "morton8":
        tile, r = i // 64, i % 64
        tiles_x = width // 8
        tx, ty = tile % tiles_x, tile // tiles_x
        lx = (r & 1) | ((r >> 1) & 2) | ((r >> 2) & 4)
        ly = ((r >> 1) & 1) | ((r >> 2) & 2) | ((r >> 3) & 4)
        return tx * 8 + lx, ty * 8 + ly
    raise ValueError(order)


def camera_rays(cam: Camera, order: str = "scanline") -> np.ndarray:
    """Primary rays at pixel centres, bit-identical to the device generator:
    u = (x + 0.5) * (1/w), v = (y + 0.5) * (1/h) in float32;
    dir = (baseDir + nearU*u) + nearV*v, each product and sum rounded once
    (PinholeCamera::getRayDirection, src/rtplugins/PinholeCamera.cpp:131-137).
    tnear = 2e-4, tfar = FLT_MAX (IAccStruct::traceNearestInstance,
    src/rtcore/IAccStruct.cpp:33-36)."""
    n = cam.width * cam.height
    px, py = camera_pixel_of_ray(np.arange(n), cam.width, cam.height, order)
    inv_w = np.float32(1.0) / np.float32(cam.width)
    inv_h = np.float32(1.0) / np.float32(cam.height)
    us = (px.astype(np.float32) + np.float32(0.5)) * inv_w
    vs = (py.astype(np.float32) + np.float32(0.5)) * inv_h
    rays = np.empty((n, RAY_WORDS), np.float32)
    rays[:, 0:3] = cam.eye
    rays[:, 3] = RAY_EPSILON
    for a in range(3):
        d = cam.base_dir[a] + cam.near_u[a] * us
        d = d + cam.near_v[a] * vs
        rays[:, 4 + a] = d
    rays[:, 7] = FLT_MAX
    return rays


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def _area2(v0, v1, v2) -> np.ndarray:
    c = np.cross((v1 - v0).astype(np.float64), (v2 - v0).astype(np.float64))
    return np.sqrt((c * c).sum(axis=1))


def random_triangles(rng, n: int, centre_lo, centre_hi, half_offset: float) -> np.ndarray:
    """n independent triangles: centroid U[lo, hi]^3, each vertex = centroid +
    U[-half_offset, half_offset]^3.  Resamples triangles whose doubled area is
    below 1e-6 * half_offset^2 (keeps every Wald record finite)."""
    lo = np.asarray(centre_lo, np.float64)
    hi = np.asarray(centre_hi, np.float64)
    out = np.empty((n, 3, 3), np.float32)
    todo = np.arange(n)
    while todo.size:
        c = rng.uniform(lo, hi, size=(todo.size, 1, 3))
        off = rng.uniform(-half_offset, half_offset, size=(todo.size, 3, 3))
        tri = (c + off).astype(np.float32)
        ok = _area2(tri[:, 0], tri[:, 1], tri[:, 2]) > 1e-6 * half_offset * half_offset
        out[todo[ok]] = tri[ok]
        todo = todo[~ok]
    return out


def plane_and_debris(seed: int = SEED_BASE + 0, quads: int = 128, debris: int = 32768) -> Scene:
    rng = _rng(seed)
    g = np.linspace(-1.0, 1.0, quads + 1, dtype=np.float64)
    zz, xx = np.meshgrid(g, g, indexing="ij")          # vertex (i=z row, j=x col)
    pv = np.stack([xx.ravel(), np.zeros(xx.size), zz.ravel()], axis=1).astype(np.float32)
    i, j = np.meshgrid(np.arange(quads), np.arange(quads), indexing="ij")
    v00 = (i * (quads + 1) + j).ravel()
    v01 = v00 + 1
    v10 = v00 + (quads + 1)
    v11 = v10 + 1
    # two triangles per quad, normal +y
    t0 = np.stack([v00, v10, v11], axis=1)
    t1 = np.stack([v00, v11, v01], axis=1)
    pidx = np.empty((2 * quads * quads, 3), np.int64)
    pidx[0::2] = t0
    pidx[1::2] = t1
    tri = random_triangles(rng, debris, (-1.0, 0.0, -1.0), (1.0, 1.0, 1.0), 0.02)
    verts = np.concatenate([pv, tri.reshape(-1, 3)], axis=0)
    didx = pv.shape[0] + np.arange(3 * debris).reshape(debris, 3)
    idx = np.concatenate([pidx, didx], axis=0).astype(np.int32)
    return Scene(verts=np.ascontiguousarray(verts), idx=np.ascontiguousarray(idx), name="plane_and_debris")


def plane_and_debris_camera(width: int = 512, height: int = 512) -> Camera:
    return look_at_camera((0.0, 1.5, 3.0), (0.0, 0.3, 0.0), (0.0, 1.0, 0.0), 60.0, width, height)


PLANE_LIGHT = np.array([2.0, 4.0, 2.0], np.float32)


def sphere_mesh(lat: int = 160, lon: int = 320):
    """Unit UV sphere, open at the poles; returns (verts, idx, normals)."""
    theta = np.pi * (np.arange(lat + 1, dtype=np.float64) + 1.0) / (lat + 2.0)
    phi = 2.0 * np.pi * np.arange(lon, dtype=np.float64) / lon
    th, ph = np.meshgrid(theta, phi, indexing="ij")
    nrm = np.stack([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)], axis=-1).reshape(-1, 3)
    verts = nrm.astype(np.float32)
    r, c = np.meshgrid(np.arange(lat), np.arange(lon), indexing="ij")
    a = r * lon + c
    b = r * lon + (c + 1) % lon
    d = (r + 1) * lon + c
    e = (r + 1) * lon + (c + 1) % lon
    idx = np.empty((lat * lon * 2, 3), np.int64)
    idx[0::2] = np.stack([a.ravel(), b.ravel(), e.ravel()], axis=1)
    idx[1::2] = np.stack([a.ravel(), e.ravel(), d.ravel()], axis=1)
    return verts, idx.astype(np.int32), nrm.astype(np.float32)


def deform(base: np.ndarray, normals: np.ndarray, frame: int) -> np.ndarray:
    """p + 0.05*sin(3*p.x + 0.3*frame)*n (host version, float64 then rounded)."""
    p = base.astype(np.float64)
    s = 0.05 * np.sin(3.0 * p[:, 0] + 0.3 * frame)
    return (p + s[:, None] * normals.astype(np.float64)).astype(np.float32)


def deforming_sphere(frame: int = 0) -> Scene:
    v, idx, n = sphere_mesh()
    return Scene(verts=deform(v, n, frame), idx=idx, name=f"deforming_sphere[{frame}]")


def deforming_sphere_camera(width: int = 1024, height: int = 1024) -> Camera:
    return look_at_camera((1.6, 1.2, 2.4), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, width, height)


SPHERE_LIGHT = np.array([3.0, 4.0, 2.0], np.float32)


def skewed_density(seed: int = SEED_BASE + 2, n: int = 1 << 20) -> Scene:
    rng = _rng(seed)
    n_small = int(round(n * 0.9))
    n_large = n - n_small
    # edge <= 2*h*sqrt(3): h = 0.00057 -> <= 0.00197 ; h = 0.144 -> <= 0.499
    small = random_triangles(rng, n_small, (-0.05,) * 3, (0.05,) * 3, 0.00057)
    large = random_triangles(rng, n_large, (-4.0,) * 3, (4.0,) * 3, 0.144)
    tri = np.concatenate([small, large], axis=0)
    perm = rng.permutation(n)
    tri = tri[perm]
    verts = tri.reshape(-1, 3)
    idx = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    return Scene(verts=np.ascontiguousarray(verts), idx=idx, name="skewed_density")


def skewed_density_camera(width: int = 1024, height: int = 1024) -> Camera:
    return look_at_camera((0.9, 0.6, 1.5), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, width, height)


def random_rays(rng, n: int, lo, hi) -> np.ndarray:
    """Rays with origins U[lo, hi]^3 and directions uniform on the sphere (no
    zero component), tnear = 2e-4, tfar = FLT_MAX."""
    o = rng.uniform(np.asarray(lo, np.float64), np.asarray(hi, np.float64), size=(n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(np.float32)
    zero = d == 0
    d[zero] = np.float32(1e-7)
    rays = np.empty((n, RAY_WORDS), np.float32)
    rays[:, 0:3] = o.astype(np.float32)
    rays[:, 3] = RAY_EPSILON
    rays[:, 4:7] = d
    rays[:, 7] = FLT_MAX
    return rays


def tiny_scene(seed: int, ntris: int, spread: float = 1.0, size: float = 0.2) -> Scene:
    """Small random soup used by unit and property tests."""
    rng = _rng(seed)
    tri = random_triangles(rng, ntris, (-spread,) * 3, (spread,) * 3, size)
    return Scene(verts=np.ascontiguousarray(tri.reshape(-1, 3)),
                 idx=np.arange(3 * ntris, dtype=np.int32).reshape(ntris, 3), name=f"tiny[{seed}]")


@dataclasses.dataclass
class BatchItem:
    scene: Scene
    rays: np.ndarray        # (R, 8) float32: primary pinhole rays first, then random rays
    n_primary: int
    camera: Camera


def batched_workload(seed: int = SEED_BASE + 3, nscenes: int = 64, tri_range=(1_000, 500_000),
                     ray_range=(4_000, 1_000_000), primary_frac: float = 0.6, order: str = "scanline"):
    """Uneven batch: scenes built like plane_and_debris with triangle counts
    log-uniform in tri_range (half ground-plane quads, half debris), each with
    a ray batch log-uniform in ray_range: primary_frac pinhole rays (square
    image, pixel centres, eye/target of the plane scene) and the rest random
    directions from uniform origins in the scene box."""
    rng = _rng(seed)
    items = []
    for i in range(nscenes):
        n_tri = int(round(math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1])))))
        quads = max(2, int(round(math.sqrt(n_tri / 4.0))))
        debris = max(1, n_tri - 2 * quads * quads)
        sc = plane_and_debris(seed=seed * 1000 + i, quads=quads, debris=debris)
        n_ray = int(round(math.exp(rng.uniform(math.log(ray_range[0]), math.log(ray_range[1])))))
        side = max(8, int(round(math.sqrt(primary_frac * n_ray) / 8.0)) * 8)
        cam = plane_and_debris_camera(side, side)
        prim = camera_rays(cam, order)
        n_rand = max(0, n_ray - prim.shape[0])
        lo = sc.verts.min(axis=0)
        hi = sc.verts.max(axis=0)
        rnd = random_rays(rng, n_rand, lo, hi)
        items.append(BatchItem(scene=sc, rays=np.ascontiguousarray(np.concatenate([prim, rnd], axis=0)),
                               n_primary=prim.shape[0], camera=cam))
    return items
