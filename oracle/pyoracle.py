"""ctypes front end of the CPU oracle.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline / reference legs -- never by the product package.

* ``liboracle.so``           the C restatement (oracle.c), built by `make` here
                             and on the GPU host.
* ``_ref/liboracle_ref.so``  the reference's own CPU sources compiled unmodified
                             (`make ref`); only present where the reference
                             checkout exists.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "liboracle_ref.so")


def reference_dir() -> str:
    """The reference checkout: GRIDRT_REFERENCE_DIR when set, else the build
    recipe's default (oracle/Makefile, `make print-ref`).  May not exist."""
    env = os.environ.get("GRIDRT_REFERENCE_DIR")
    if env:
        return env
    try:
        out = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True, timeout=60)
        return out.stdout.strip()
    except Exception:
        return ""


_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


class GridInfo(C.Structure):
    _fields_ = [("res", C.c_int32 * 3), ("bmin", C.c_float * 3), ("bmax", C.c_float * 3),
                ("cell", C.c_float * 3), ("inv_cell", C.c_float * 3), ("ncells", C.c_int64),
                ("nrefs", C.c_int64)]

    def as_dict(self):
        return dict(res=tuple(self.res), bmin=np.array(self.bmin, np.float32), bmax=np.array(self.bmax, np.float32),
                    cell=np.array(self.cell, np.float32), inv_cell=np.array(self.inv_cell, np.float32),
                    ncells=int(self.ncells), nrefs=int(self.nrefs))


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and, with ref=True, the compiled reference when its
    sources are present)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    ref_src = reference_dir() if ref else ""
    if ref_src and os.path.isdir(os.path.join(ref_src, "src", "rtplugins")):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF={ref_src}"])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_grid_params.argtypes = [_f32p, C.c_int64, C.c_int64, C.c_int32, C.POINTER(GridInfo)]
        L.orc_grid_build.argtypes = [_f32p, C.c_int64, _i32p, C.c_int64, C.c_int32, C.POINTER(GridInfo),
                                     C.c_void_p, C.c_void_p]
        L.orc_triaccel_build.argtypes = [_f32p, _i32p, C.c_int64, _f32p]
        L.orc_trace_closest.argtypes = [C.POINTER(GridInfo), _i32p, _i32p, _f32p, _f32p, C.c_int64, _f32p,
                                        C.c_void_p, C.c_int]
        L.orc_trace_any.argtypes = [C.POINTER(GridInfo), _i32p, _i32p, _f32p, _f32p, C.c_int64, _u8p,
                                    C.c_void_p, C.c_int]
        L.orc_mt_f64.argtypes = [_f32p, _i32p, _f32p, _i32p, C.c_int64, _f64p]
        L.orc_max_threads.restype = C.c_int
        L.orc_instance_box.argtypes = [_f32p, _f32p, _f32p, _f32p, _f32p]
        L.orc_scene_box.argtypes = [C.c_int32, _f32p, _f32p]
        L.orc_trace_instances.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, _f32p, _f32p,
                                          _f32p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        _lib = L
    return _lib


def max_threads() -> int:
    return int(lib().orc_max_threads())


class Grid:
    """Oracle grid for one scene (restatement of the reference builder)."""

    def __init__(self, verts: np.ndarray, idx: np.ndarray, k: int):
        self.verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        self.idx = np.ascontiguousarray(idx, np.int32).reshape(-1, 3)
        self.k = int(k)
        info = GridInfo()
        L = lib()
        rc = L.orc_grid_build(self.verts.ravel(), self.verts.shape[0], self.idx.ravel(), self.idx.shape[0],
                              self.k, C.byref(info), None, None)
        if rc:
            raise ValueError(f"oracle grid build failed ({rc})")
        self.offsets = np.empty(info.ncells + 1, np.int32)
        self.ids = np.empty(max(info.nrefs, 1), np.int32)
        rc = L.orc_grid_build(self.verts.ravel(), self.verts.shape[0], self.idx.ravel(), self.idx.shape[0],
                              self.k, C.byref(info), self.offsets.ctypes.data, self.ids.ctypes.data)
        if rc:
            raise ValueError(f"oracle grid build failed ({rc})")
        self.ids = self.ids[:info.nrefs]
        self.info = info
        self.acc = np.empty((self.idx.shape[0], 12), np.float32)
        L.orc_triaccel_build(self.verts.ravel(), self.idx.ravel(), self.idx.shape[0], self.acc.ravel())

    @property
    def ids_padded(self):
        return self.ids if self.ids.size else np.zeros(1, np.int32)

    def trace_closest(self, rays: np.ndarray, counters: bool = False, nthreads: int = 0):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        hits = np.empty((n, 4), np.float32)
        cnt = np.empty((n, 2), np.int64) if counters else None
        lib().orc_trace_closest(C.byref(self.info), self.offsets, self.ids_padded, self.acc.ravel(), rays.ravel(),
                                n, hits.ravel(), cnt.ctypes.data if counters else None, int(nthreads))
        return (split_hits(hits), cnt) if counters else split_hits(hits)

    def trace_any(self, rays: np.ndarray, counters: bool = False, nthreads: int = 0):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        occ = np.empty(n, np.uint8)
        cnt = np.empty((n, 2), np.int64) if counters else None
        lib().orc_trace_any(C.byref(self.info), self.offsets, self.ids_padded, self.acc.ravel(), rays.ravel(), n,
                            occ, cnt.ctypes.data if counters else None, int(nthreads))
        return (occ, cnt) if counters else occ


class Material(C.Structure):
    _fields_ = [("type", C.c_int32), ("ambient", C.c_float * 3), ("diffuse", C.c_float * 3),
                ("specular", C.c_float * 3), ("specular_exponent", C.c_float), ("reflexion", C.c_float),
                ("refraction_index", C.c_float), ("opacity", C.c_float)]


class Light(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("intensity", C.c_float * 3), ("cast_shadows", C.c_int32),
                ("pad", C.c_int32)]


def render(grid: "Grid", normals, colors, material, mats, lights, background, max_depth, medium, primary,
           nthreads: int = 0):
    """Restated per-pixel shading recursion -> (rgb (n, 3) float32, rays traced)."""
    primary = np.ascontiguousarray(primary, np.float32).reshape(-1, 8)
    n = primary.shape[0]
    rgb = np.empty((n, 3), np.float32)
    normals = np.ascontiguousarray(normals, np.float32)
    colors = None if colors is None else np.ascontiguousarray(colors, np.float32)
    material = None if material is None else np.ascontiguousarray(material, np.int32)
    M = (Material * max(1, len(mats)))(*mats)
    Lt = (Light * max(1, len(lights)))(*lights)
    bg = np.ascontiguousarray(background, np.float32)
    L = lib()
    L.orc_render.restype = C.c_int64
    L.orc_render.argtypes = [C.POINTER(GridInfo), _i32p, _i32p, _f32p, _i32p, _f32p, C.c_void_p, C.c_void_p,
                             C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, _f32p, C.c_int32, C.c_float, _f32p,
                             C.c_int64, _f32p, C.c_int]
    total = L.orc_render(C.byref(grid.info), grid.offsets, grid.ids_padded, grid.acc.ravel(), grid.idx.ravel(),
                         normals.ravel(), None if colors is None else colors.ctypes.data,
                         None if material is None else material.ctypes.data, C.cast(M, C.c_void_p), len(mats),
                         C.cast(Lt, C.c_void_p), len(lights), bg, int(max_depth), float(medium), primary.ravel(), n,
                         rgb.ravel(), int(nthreads))
    return rgb, int(total)


class Instances:
    """Oracle instance set: (Grid, world_from_local 3x4, local_from_world 3x4)
    triples, restating Context::instantiateGeometry, buildInstance and
    traceNearestInstance (see oracle.c)."""

    def __init__(self, items):
        self.items = [(g, np.ascontiguousarray(xf, np.float32).reshape(12), np.ascontiguousarray(inv, np.float32)
                       .reshape(12)) for g, xf, inv in items]
        L = lib()
        n = len(self.items)
        self.boxes = np.empty((n, 6), np.float32)
        for i, (g, xf, _) in enumerate(self.items):
            bmin = np.ascontiguousarray(g.info.bmin, np.float32)
            bmax = np.ascontiguousarray(g.info.bmax, np.float32)
            lo = np.empty(3, np.float32)
            hi = np.empty(3, np.float32)
            L.orc_instance_box(bmin, bmax, xf, lo, hi)
            self.boxes[i, :3] = lo
            self.boxes[i, 3:] = hi
        self.box = np.empty(6, np.float32)
        L.orc_scene_box(n, self.boxes.ravel(), self.box)
        self._g = (C.POINTER(GridInfo) * n)(*[C.pointer(g.info) for g, _, _ in self.items])
        self._off = (C.c_void_p * n)(*[g.offsets.ctypes.data for g, _, _ in self.items])
        self._ids = (C.c_void_p * n)(*[g.ids_padded.ctypes.data for g, _, _ in self.items])
        self._acc = (C.c_void_p * n)(*[g.acc.ctypes.data for g, _, _ in self.items])
        self._inv = np.ascontiguousarray(np.stack([inv for _, _, inv in self.items]), np.float32).ravel()

    def trace(self, rays: np.ndarray, nthreads: int = 0):
        """-> (hits dict, instance index per ray, occluded per ray)."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        hits = np.empty((n, 4), np.float32)
        inst = np.empty(n, np.int32)
        occ = np.empty(n, np.uint8)
        lib().orc_trace_instances(len(self.items), C.cast(self._g, C.c_void_p), C.cast(self._off, C.c_void_p),
                                  C.cast(self._ids, C.c_void_p), C.cast(self._acc, C.c_void_p), self._inv, self.box,
                                  rays.ravel(), n, hits.ctypes.data, inst.ctypes.data, occ.ctypes.data,
                                  int(nthreads))
        return split_hits(hits), inst, occ


def grid_params(verts: np.ndarray, ntris: int, k: int) -> dict:
    verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
    info = GridInfo()
    rc = lib().orc_grid_params(verts.ravel(), verts.shape[0], int(ntris), int(k), C.byref(info))
    if rc:
        raise ValueError("empty input")
    return info.as_dict()


def split_hits(hits: np.ndarray) -> dict:
    hits = np.ascontiguousarray(hits, np.float32).reshape(-1, 4)
    return dict(id=hits[:, 0].copy().view(np.int32), t=hits[:, 1].copy(), u=hits[:, 2].copy(), v=hits[:, 3].copy())


def mt_f64(verts, idx, rays, tri) -> np.ndarray:
    verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(idx, np.int32).reshape(-1, 3)
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    tri = np.ascontiguousarray(tri, np.int32)
    out = np.empty((tri.shape[0], 3), np.float64)
    lib().orc_mt_f64(verts.ravel(), idx.ravel(), rays.ravel(), tri, tri.shape[0], out.ravel())
    return out


# ---- the reference's own code (compiled from its sources) --------------------

_ref = None


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_PATH)
        L.ref_scene_create.restype = C.c_void_p
        L.ref_scene_create.argtypes = [_f32p, C.c_int64, _i32p, C.c_int64, C.c_int]
        L.ref_scene_destroy.argtypes = [C.c_void_p]
        L.ref_scene_grid_info.argtypes = [C.c_void_p, _i32p, _f32p, _f32p, _f32p, _i64p]
        L.ref_scene_grid_csr.argtypes = [C.c_void_p, _i32p, _i32p]
        L.ref_scene_trace.argtypes = [C.c_void_p, _f32p, C.c_int64, _f32p, C.c_int, C.c_int]
        L.ref_scene_triaccel.argtypes = [C.c_void_p, _f32p]
        _ref = L
    return _ref


class RefScene:
    """The reference's UniformGridAccStructBuilder + UniformGridAccStruct
    (k = 6, as hard-coded at src/rtplugins/UniformGridAccStructBuilder.cpp:91)."""

    K = 6

    def __init__(self, verts, idx, quiet: bool = True):
        self.verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        self.idx = np.ascontiguousarray(idx, np.int32).reshape(-1, 3)
        L = ref_lib()
        self.h = L.ref_scene_create(self.verts.ravel(), self.verts.shape[0], self.idx.ravel(), self.idx.shape[0],
                                    1 if quiet else 0)
        if not self.h:
            raise ValueError("reference rejected the geometry (invalid triangle or index)")
        res = np.zeros(3, np.int32)
        bbox = np.zeros(6, np.float32)
        cell = np.zeros(3, np.float32)
        inv = np.zeros(3, np.float32)
        nrefs = np.zeros(1, np.int64)
        L.ref_scene_grid_info(self.h, res, bbox, cell, inv, nrefs)
        self.info = dict(res=tuple(int(r) for r in res), bmin=bbox[:3].copy(), bmax=bbox[3:].copy(), cell=cell,
                         inv_cell=inv, ncells=int(np.prod(res.astype(np.int64))), nrefs=int(nrefs[0]))

    def csr(self):
        off = np.empty(self.info["ncells"] + 1, np.int32)
        ids = np.empty(max(self.info["nrefs"], 1), np.int32)
        ref_lib().ref_scene_grid_csr(self.h, off, ids)
        return off, ids[:self.info["nrefs"]]

    def triaccel(self):
        out = np.empty((self.idx.shape[0], 12), np.float32)
        ref_lib().ref_scene_triaccel(self.h, out.ravel())
        return out

    def trace(self, rays, brute: bool = False, nthreads: int = 0):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        hits = np.empty((rays.shape[0], 4), np.float32)
        ref_lib().ref_scene_trace(self.h, rays.ravel(), rays.shape[0], hits.ravel(), 1 if brute else 0, int(nthreads))
        return split_hits(hits)

    def __del__(self):
        if getattr(self, "h", None) and _ref is not None:
            _ref.ref_scene_destroy(self.h)
            self.h = None
