"""ctypes binding of libgridrt.so (the C ABI in include/gridrt.h).

This module is plumbing for Python callers (tests, bench): every compute call
goes through the CUDA library.  Loading fails loudly when the library is
missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

RTG_OK = 0
RTG_NO_MEMORY = 1
RTG_INVALID_PARAM = 3
RTG_DEVICE_ERROR = 4
RTG_TIMEOUT = 5
RTG_NOT_BUILT = 6
RTG_INVALID_GEOMETRY = 7

RTG_TRACE_COUNTERS = 1
RTG_TUNE_EMPTY_RUN = 1
RTG_TUNE_PERSISTENT = 2
RTG_TUNE_CELL_RECORDS = 3
RTG_TUNE_BLOCK = 7
RTG_TUNE_LANES = 8
RTG_TUNE_HEAVY_CELL = 4
RTG_TUNE_HEAVY_LANES = 5
RTG_TUNE_REFILL = 6
ORDER = {"scanline": 0, "morton8": 1}


class GridRTError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"gridrt status {status}: {msg}")
        self.status = status


class GridInfo(C.Structure):
    _fields_ = [("res", C.c_int32 * 3), ("bmin", C.c_float * 3), ("bmax", C.c_float * 3), ("cell", C.c_float * 3),
                ("inv_cell", C.c_float * 3), ("ncells", C.c_int64), ("nrefs", C.c_int64), ("k", C.c_int32),
                ("built", C.c_int32)]

    def as_dict(self):
        return dict(res=tuple(self.res), bmin=np.array(self.bmin, np.float32), bmax=np.array(self.bmax, np.float32),
                    cell=np.array(self.cell, np.float32), inv_cell=np.array(self.inv_cell, np.float32),
                    ncells=int(self.ncells), nrefs=int(self.nrefs), k=int(self.k), built=bool(self.built))


class TraceTaskC(C.Structure):
    _fields_ = [("scene", C.c_int32), ("mode", C.c_int32), ("d_rays", C.c_void_p), ("n", C.c_int64),
                ("d_out", C.c_void_p)]


class RequestC(C.Structure):
    _fields_ = [("arrival_s", C.c_double), ("scene", C.c_int32), ("mode", C.c_int32), ("h_rays", C.c_void_p),
                ("n", C.c_int64), ("h_out", C.c_void_p)]


class RequestTimesC(C.Structure):
    _fields_ = [("admit_s", C.c_double), ("done_s", C.c_double)]


class ServeOptionsC(C.Structure):
    _fields_ = [("pool_bytes", C.c_int64), ("max_step_rays", C.c_int64), ("max_in_flight", C.c_int32),
                ("plain", C.c_int32), ("empty_run", C.c_int32), ("pad", C.c_int32)]


class InstanceC(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("world_from_local", C.c_float * 12), ("local_from_world", C.c_float * 12)]


class MaterialC(C.Structure):
    _fields_ = [("type", C.c_int32), ("ambient", C.c_float * 3), ("diffuse", C.c_float * 3),
                ("specular", C.c_float * 3), ("specular_exponent", C.c_float), ("reflexion", C.c_float),
                ("refraction_index", C.c_float), ("opacity", C.c_float)]


class PointLightC(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("intensity", C.c_float * 3), ("cast_shadows", C.c_int32),
                ("pad", C.c_int32)]


class ShadingC(C.Structure):
    _fields_ = [("d_normals", C.c_void_p), ("d_colors", C.c_void_p), ("d_material", C.c_void_p),
                ("materials", C.POINTER(MaterialC)), ("nmaterials", C.c_int32),
                ("lights", C.POINTER(PointLightC)), ("nlights", C.c_int32), ("background", C.c_float * 3),
                ("max_depth", C.c_int32), ("medium_index", C.c_float)]


RTG_MAT_HEADLIGHT, RTG_MAT_HEADLIGHT_COLOR, RTG_MAT_PHONG, RTG_MAT_PHONG_COLOR = 0, 1, 2, 3


def material(type=RTG_MAT_PHONG, ambient=(0.2, 0.2, 0.2), diffuse=(1, 1, 1), specular=(1, 1, 1),
             specular_exponent=32.0, reflexion=0.0, refraction_index=1.0, opacity=1.0) -> MaterialC:
    """Defaults of PhongMaterial (src/rtplugins/PhongMaterial.cpp:8-17)."""
    m = MaterialC()
    m.type = type
    for a in range(3):
        m.ambient[a], m.diffuse[a], m.specular[a] = ambient[a], diffuse[a], specular[a]
    m.specular_exponent, m.reflexion, m.refraction_index, m.opacity = (specular_exponent, reflexion,
                                                                        refraction_index, opacity)
    return m


def point_light(position, intensity=(1, 1, 1), cast_shadows=True) -> PointLightC:
    L = PointLightC()
    for a in range(3):
        L.position[a], L.intensity[a] = position[a], intensity[a]
    L.cast_shadows = 1 if cast_shadows else 0
    return L


class MeshC(C.Structure):
    _fields_ = [("verts", C.POINTER(C.c_float)), ("nverts", C.c_int64), ("tris", C.POINTER(C.c_int32)),
                ("ntris", C.c_int64), ("source_face", C.POINTER(C.c_int64)), ("faces", C.c_int64),
                ("dropped", C.c_int64)]


class CameraC(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("base_dir", C.c_float * 3), ("near_u", C.c_float * 3),
                ("near_v", C.c_float * 3), ("width", C.c_int32), ("height", C.c_int32), ("order", C.c_int32),
                ("pad", C.c_int32)]


def camera_struct(cam, order: str = "scanline") -> CameraC:
    c = CameraC()
    for a in range(3):
        c.eye[a] = float(cam.eye[a])
        c.base_dir[a] = float(cam.base_dir[a])
        c.near_u[a] = float(cam.near_u[a])
        c.near_v[a] = float(cam.near_v[a])
    c.width, c.height, c.order = int(cam.width), int(cam.height), ORDER[order]
    return c


_lib = None
EXPORTS = [
    "rtg_version", "rtg_last_error", "rtg_scene_create", "rtg_scene_destroy", "rtg_scene_stream",
    "rtg_scene_set_geometry", "rtg_scene_set_geometry_device", "rtg_scene_update_vertices",
    "rtg_scene_deform_vertices", "rtg_scene_build", "rtg_scene_build_async", "rtg_scene_build_check",
    "rtg_scene_reserve", "rtg_scene_grid_info", "rtg_scene_grid_download", "rtg_scene_download_vertices", "rtg_scene_grid_device",
    "rtg_trace_nearest", "rtg_trace_nearest_device", "rtg_trace_any", "rtg_trace_any_device",
    "rtg_trace_camera_device", "rtg_trace_camera_diffuse_device", "rtg_trace_frame_device", "rtg_trace_frame",
    "rtg_trace_frame_async", "rtg_trace_frame_wait", "rtg_grid_build_noalloc",
    "rtg_kernel_launch_count",
    "rtg_scene_set_tuning", "rtg_scene_counters", "rtg_batch_create", "rtg_batch_build_async",
    "rtg_batch_trace_async", "rtg_batch_check", "rtg_batch_rays", "rtg_batch_set_tuning", "rtg_batch_destroy",
    "rtg_serve_run",
    "rtg_instances_create", "rtg_instances_update", "rtg_instances_box", "rtg_instances_set_tuning",
    "rtg_trace_nearest_instances_device", "rtg_trace_any_instances_device", "rtg_trace_nearest_instances",
    "rtg_instances_destroy", "rtg_probe_read_gbs",
    "rtg_mesh_load", "rtg_mesh_free", "rtg_scene_load", "rtg_scene_stage_vertices", "rtg_render",
]


def lib_path() -> str:
    """The in-tree library; GRIDRT_LIB names another build of the same
    sources (e.g. one compiled with different -D options)."""
    return os.environ.get("GRIDRT_LIB") or _build.LIB


def load(build_if_missing: bool = True):
    """Load libgridrt.so (building it when absent and allowed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise FileNotFoundError(f"{path} missing: run __graft_entry__.build()")
        _build.build()
    L = C.CDLL(path)
    vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int32
    sig = {
        "rtg_version": ([], C.c_char_p),
        "rtg_last_error": ([], C.c_char_p),
        "rtg_scene_create": ([C.c_int, vp, C.POINTER(vp)], C.c_int),
        "rtg_scene_destroy": ([vp], C.c_int),
        "rtg_scene_stream": ([vp, C.POINTER(vp)], C.c_int),
        "rtg_scene_set_geometry": ([vp, vp, i64, vp, i64, vp], C.c_int),
        "rtg_scene_set_geometry_device": ([vp, vp, i64, vp, i64, vp], C.c_int),
        "rtg_scene_update_vertices": ([vp, vp, i64, C.c_int, vp], C.c_int),
        "rtg_scene_deform_vertices": ([vp, vp, vp, C.c_float, C.c_float, C.c_float, vp], C.c_int),
        "rtg_scene_build": ([vp, i32, vp], C.c_int),
        "rtg_scene_build_async": ([vp, i32, vp], C.c_int),
        "rtg_scene_build_check": ([vp, vp], C.c_int),
        "rtg_scene_reserve": ([vp, i64, i64], C.c_int),
        "rtg_scene_grid_info": ([vp, C.POINTER(GridInfo)], C.c_int),
        "rtg_scene_grid_download": ([vp, vp, vp], C.c_int),
        "rtg_scene_download_vertices": ([vp, vp], C.c_int),
        "rtg_scene_grid_device": ([vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)], C.c_int),
        "rtg_trace_nearest": ([vp, vp, i64, vp, i32, vp], C.c_int),
        "rtg_trace_nearest_device": ([vp, vp, i64, vp, i32, vp], C.c_int),
        "rtg_trace_any": ([vp, vp, i64, vp, i32, vp], C.c_int),
        "rtg_trace_any_device": ([vp, vp, i64, vp, i32, vp], C.c_int),
        "rtg_trace_camera_device": ([vp, C.POINTER(CameraC), vp, vp, vp, i32, vp], C.c_int),
        "rtg_trace_camera_diffuse_device": ([vp, C.POINTER(CameraC), C.c_uint64, vp, vp, i32, vp], C.c_int),
        "rtg_trace_frame_device": ([vp, C.POINTER(CameraC), vp, vp, vp, vp, vp], C.c_int),
        "rtg_trace_frame": ([vp, C.POINTER(CameraC), vp, vp, vp, vp], C.c_int),
        "rtg_trace_frame_async": ([vp, C.POINTER(CameraC), vp, vp, vp, vp, C.POINTER(C.c_uint64)], C.c_int),
        "rtg_trace_frame_wait": ([vp, C.c_uint64], C.c_int),
        "rtg_grid_build_noalloc": ([vp, i64, vp, i64, i32, vp, i64, vp, i64, vp, C.POINTER(GridInfo), vp],
                                   C.c_int),
        "rtg_kernel_launch_count": ([], C.c_uint64),
        "rtg_scene_set_tuning": ([vp, i32, i32], C.c_int),
        "rtg_batch_create": ([C.POINTER(vp), i32, C.POINTER(i32), C.POINTER(TraceTaskC), i32, C.POINTER(vp)],
                             C.c_int),
        "rtg_batch_build_async": ([vp, vp], C.c_int),
        "rtg_batch_trace_async": ([vp, vp], C.c_int),
        "rtg_batch_check": ([vp, vp], C.c_int),
        "rtg_batch_rays": ([vp, C.POINTER(i64)], C.c_int),
        "rtg_batch_set_tuning": ([vp, i32, i32], C.c_int),
        "rtg_batch_destroy": ([vp], C.c_int),
        "rtg_serve_run": ([C.POINTER(vp), i32, C.POINTER(RequestC), i64, C.POINTER(ServeOptionsC),
                           C.POINTER(RequestTimesC)], C.c_int),
        "rtg_scene_counters": ([vp, C.POINTER(C.c_int64), C.c_int], C.c_int),
        "rtg_instances_create": ([C.POINTER(InstanceC), i32, C.POINTER(vp)], C.c_int),
        "rtg_instances_update": ([vp, C.POINTER(InstanceC), i32], C.c_int),
        "rtg_instances_box": ([vp, vp, vp], C.c_int),
        "rtg_instances_set_tuning": ([vp, i32, i32], C.c_int),
        "rtg_trace_nearest_instances_device": ([vp, vp, i64, vp, vp, i32, vp], C.c_int),
        "rtg_trace_any_instances_device": ([vp, vp, i64, vp, i32, vp], C.c_int),
        "rtg_trace_nearest_instances": ([vp, vp, i64, vp, vp, vp], C.c_int),
        "rtg_instances_destroy": ([vp], C.c_int),
        "rtg_probe_read_gbs": ([i32, i64, i32, C.POINTER(C.c_double)], C.c_int),
        "rtg_mesh_load": ([C.c_char_p, C.POINTER(MeshC)], C.c_int),
        "rtg_mesh_free": ([C.POINTER(MeshC)], None),
        "rtg_scene_load": ([vp, C.c_char_p, C.POINTER(MeshC)], C.c_int),
        "rtg_scene_stage_vertices": ([vp, vp, i64, vp], C.c_int),
        "rtg_render": ([vp, C.POINTER(CameraC), C.POINTER(ShadingC), vp, C.POINTER(C.c_int64), vp], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def check(rc: int):
    if rc != RTG_OK:
        raise GridRTError(rc, load().rtg_last_error().decode())


def _ptr(a) -> int:
    """Address of a numpy array or torch tensor (an int is taken as an address)."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


class Scene:
    """One geometry with its device-resident uniform grid."""

    def __init__(self, device: int = 0, stream=None):
        L = load()
        h = C.c_void_p()
        check(L.rtg_scene_create(int(device), stream, C.byref(h)))
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            load().rtg_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        check(load().rtg_scene_stream(self.h, C.byref(s)))
        return s.value or 0

    # ---- geometry -----------------------------------------------------------
    def set_geometry(self, verts: np.ndarray, idx: np.ndarray):
        self._verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        self._idx = np.ascontiguousarray(idx, np.int32).reshape(-1, 3)
        self._nverts = self._verts.shape[0]
        check(load().rtg_scene_set_geometry(self.h, _ptr(self._verts), self._verts.shape[0], _ptr(self._idx),
                                            self._idx.shape[0], None))

    def set_geometry_device(self, d_verts, nverts: int, d_idx, ntris: int, stream=None):
        self._nverts = int(nverts)
        check(load().rtg_scene_set_geometry_device(self.h, _ptr(d_verts), nverts, _ptr(d_idx), ntris, stream))

    def update_vertices(self, verts, nverts: int, from_device: bool, stream=None):
        check(load().rtg_scene_update_vertices(self.h, _ptr(verts), nverts, 1 if from_device else 0, stream))

    def deform(self, d_base, d_normals, amp: float, freq: float, phase: float, stream=None):
        check(load().rtg_scene_deform_vertices(self.h, _ptr(d_base), _ptr(d_normals), amp, freq, phase, stream))

    # ---- grid ---------------------------------------------------------------
    def load(self, path: str) -> dict:
        m = MeshC()
        check(load().rtg_scene_load(self.h, str(path).encode(), C.byref(m)))
        info = dict(nverts=int(m.nverts), ntris=int(m.ntris), faces=int(m.faces), dropped=int(m.dropped))
        load().rtg_mesh_free(C.byref(m))
        self._nverts = info["nverts"]
        return info

    def render(self, cam, d_normals, materials, lights, d_rgb, d_colors=None, d_material=None,
               background=(1.0, 1.0, 1.0), max_depth: int = 3, medium_index: float = 1.0, stream=None) -> int:
        """Shading wavefront (rtg_render) into d_rgb (H*W*3 float32); returns rays traced."""
        sh = ShadingC()
        sh.d_normals = _ptr(d_normals)
        sh.d_colors = _ptr(d_colors) if d_colors is not None else None
        sh.d_material = _ptr(d_material) if d_material is not None else None
        mats = (MaterialC * max(1, len(materials)))(*materials)
        lts = (PointLightC * max(1, len(lights)))(*lights)
        sh.materials = mats
        sh.nmaterials = len(materials)
        sh.lights = lts
        sh.nlights = len(lights)
        for a in range(3):
            sh.background[a] = background[a]
        sh.max_depth = max_depth
        sh.medium_index = medium_index
        cs = camera_struct(cam, "scanline")
        rays = C.c_int64()
        check(load().rtg_render(self.h, C.byref(cs), C.byref(sh), _ptr(d_rgb), C.byref(rays), stream))
        return rays.value

    def stage_vertices(self, host_verts, nverts: int, copy_stream=None):
        """Double-buffered keyframe upload (pinned host memory)."""
        check(load().rtg_scene_stage_vertices(self.h, _ptr(host_verts), int(nverts), copy_stream))

    def build(self, k: int, stream=None):
        check(load().rtg_scene_build(self.h, int(k), stream))

    def build_async(self, k: int, stream=None):
        check(load().rtg_scene_build_async(self.h, int(k), stream))

    def build_check(self, stream=None) -> int:
        return load().rtg_scene_build_check(self.h, stream)

    def reserve(self, ncells: int, nrefs: int):
        check(load().rtg_scene_reserve(self.h, int(ncells), int(nrefs)))

    def info(self) -> dict:
        gi = GridInfo()
        check(load().rtg_scene_grid_info(self.h, C.byref(gi)))
        return gi.as_dict()

    def download(self):
        inf = self.info()
        off = np.empty(inf["ncells"] + 1, np.int32)
        ids = np.empty(max(inf["nrefs"], 1), np.int32)
        check(load().rtg_scene_grid_download(self.h, _ptr(off), _ptr(ids)))
        return off, ids[:inf["nrefs"]]

    def download_vertices(self) -> np.ndarray:
        n = getattr(self, "_nverts", 0)
        out = np.empty((n, 3), np.float32)
        check(load().rtg_scene_download_vertices(self.h, _ptr(out)))
        return out

    def device_arrays(self):
        o, i, t = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(load().rtg_scene_grid_device(self.h, C.byref(o), C.byref(i), C.byref(t)))
        return o.value, i.value, t.value

    # ---- tracing ------------------------------------------------------------
    def trace_nearest(self, rays: np.ndarray, counters: bool = False) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        hits = np.empty((rays.shape[0], 4), np.float32)
        check(load().rtg_trace_nearest(self.h, _ptr(rays), rays.shape[0], _ptr(hits),
                                       RTG_TRACE_COUNTERS if counters else 0, None))
        return hits

    def trace_any(self, rays: np.ndarray, counters: bool = False) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        occ = np.empty(rays.shape[0], np.uint8)
        check(load().rtg_trace_any(self.h, _ptr(rays), rays.shape[0], _ptr(occ),
                                   RTG_TRACE_COUNTERS if counters else 0, None))
        return occ

    def trace_nearest_device(self, d_rays, n: int, d_hits, counters: bool = False, stream=None):
        check(load().rtg_trace_nearest_device(self.h, _ptr(d_rays), int(n), _ptr(d_hits),
                                              RTG_TRACE_COUNTERS if counters else 0, stream))

    def trace_any_device(self, d_rays, n: int, d_occ, counters: bool = False, stream=None):
        check(load().rtg_trace_any_device(self.h, _ptr(d_rays), int(n), _ptr(d_occ),
                                          RTG_TRACE_COUNTERS if counters else 0, stream))

    def trace_camera_device(self, cam, d_hits, light=None, d_shadow_rays=None, order: str = "scanline",
                            counters: bool = False, stream=None):
        cs = camera_struct(cam, order)
        lp = None
        if light is not None:
            self._light = np.ascontiguousarray(light, np.float32)
            lp = _ptr(self._light)
        check(load().rtg_trace_camera_device(self.h, C.byref(cs), _ptr(d_hits), lp, _ptr(d_shadow_rays),
                                             RTG_TRACE_COUNTERS if counters else 0, stream))

    def trace_camera_diffuse_device(self, cam, seed: int, d_hits, d_secondary, order: str = "scanline",
                                    counters: bool = False, stream=None):
        cs = camera_struct(cam, order)
        check(load().rtg_trace_camera_diffuse_device(self.h, C.byref(cs), int(seed), _ptr(d_hits), _ptr(d_secondary),
                                                     RTG_TRACE_COUNTERS if counters else 0, stream))

    def trace_frame_device(self, cam, light, d_hits, d_occ, d_shadow_rays, order: str = "scanline", stream=None):
        cs = camera_struct(cam, order)
        self._light = np.ascontiguousarray(light, np.float32)
        check(load().rtg_trace_frame_device(self.h, C.byref(cs), _ptr(self._light), _ptr(d_hits), _ptr(d_occ),
                                            _ptr(d_shadow_rays), stream))

    def trace_frame(self, cam, light, hits_host, occ_host, order: str = "scanline", stream=None):
        """Primary + shadow frame with host outputs (pinned buffers copy fastest)."""
        cs = camera_struct(cam, order)
        self._light = np.ascontiguousarray(light, np.float32)
        check(load().rtg_trace_frame(self.h, C.byref(cs), _ptr(self._light), _ptr(hits_host), _ptr(occ_host),
                                     stream))

    def trace_frame_async(self, cam, light, hits_host, occ_host, order: str = "scanline", stream=None) -> int:
        """trace_frame without waiting: returns the frame's ticket; the host
        buffers (pinned, kept alive by the caller) are complete after
        trace_frame_wait(ticket)."""
        cs = camera_struct(cam, order)
        self._light = np.ascontiguousarray(light, np.float32)
        t = C.c_uint64(0)
        check(load().rtg_trace_frame_async(self.h, C.byref(cs), _ptr(self._light), _ptr(hits_host), _ptr(occ_host),
                                           stream, C.byref(t)))
        return int(t.value)

    def trace_frame_wait(self, ticket: int):
        check(load().rtg_trace_frame_wait(self.h, int(ticket)))

    def set_tuning(self, empty_run: int = None, persistent: bool = None, cell_records: bool = None,
                   heavy_cell: int = None, heavy_lanes: int = None, refill: int = None, block: int = None,
                   lanes: int = None):
        if block is not None:
            check(load().rtg_scene_set_tuning(self.h, RTG_TUNE_BLOCK, int(block)))
        if lanes is not None:
            check(load().rtg_scene_set_tuning(self.h, RTG_TUNE_LANES, int(lanes)))
        if empty_run is not None:
            check(load().rtg_scene_set_tuning(self.h, RTG_TUNE_EMPTY_RUN, int(empty_run)))
        if persistent is not None:
            check(load().rtg_scene_set_tuning(self.h, RTG_TUNE_PERSISTENT, 1 if persistent else 0))
        if cell_records is not None:
            check(load().rtg_scene_set_tuning(self.h, RTG_TUNE_CELL_RECORDS, 1 if cell_records else 0))
        if heavy_cell is not None:
            check(load().rtg_scene_set_tuning(self.h, RTG_TUNE_HEAVY_CELL, int(heavy_cell)))
        if heavy_lanes is not None:
            check(load().rtg_scene_set_tuning(self.h, RTG_TUNE_HEAVY_LANES, int(heavy_lanes)))
        if refill is not None:
            check(load().rtg_scene_set_tuning(self.h, RTG_TUNE_REFILL, int(refill)))

    def counters(self, reset: bool = True):
        out = (C.c_int64 * 3)()
        check(load().rtg_scene_counters(self.h, out, 1 if reset else 0))
        return dict(rays=out[0], cells=out[1], tests=out[2])


RTG_MODE_NEAREST = 0
RTG_MODE_ANY = 1


def _instance_structs(items):
    arr = (InstanceC * len(items))()
    for i, (scene, xf, inv) in enumerate(items):
        arr[i].scene = scene.h
        xf = np.ascontiguousarray(xf, np.float32).reshape(12)
        inv = np.ascontiguousarray(inv, np.float32).reshape(12)
        for k in range(12):
            arr[i].world_from_local[k] = float(xf[k])
            arr[i].local_from_world[k] = float(inv[k])
    return arr


class Instances:
    """Ordered instance set over built scenes: (Scene, world_from_local 3x4,
    local_from_world 3x4) triples (rtg_instances_*)."""

    def __init__(self, items):
        self.items = list(items)
        h = C.c_void_p()
        arr = _instance_structs(self.items)
        check(load().rtg_instances_create(arr, len(self.items), C.byref(h)))
        self.h = h

    def update(self, items):
        self.items = list(items)
        arr = _instance_structs(self.items)
        check(load().rtg_instances_update(self.h, arr, len(self.items)))

    def boxes(self):
        box = np.empty(6, np.float32)
        inst = np.empty((len(self.items), 6), np.float32)
        check(load().rtg_instances_box(self.h, _ptr(box), _ptr(inst)))
        return box, inst

    def set_tuning(self, empty_run: int = None, persistent: bool = None):
        if empty_run is not None:
            check(load().rtg_instances_set_tuning(self.h, RTG_TUNE_EMPTY_RUN, int(empty_run)))
        if persistent is not None:
            check(load().rtg_instances_set_tuning(self.h, RTG_TUNE_PERSISTENT, 1 if persistent else 0))

    def trace_nearest(self, rays: np.ndarray):
        """Host rays -> (n x 4 hit words, instance index per ray)."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        hits = np.empty((n, 4), np.float32)
        inst = np.empty(n, np.int32)
        check(load().rtg_trace_nearest_instances(self.h, _ptr(rays), n, _ptr(hits), _ptr(inst), None))
        return hits, inst

    def trace_nearest_device(self, d_rays, n: int, d_hits, d_inst=None, stream=None):
        check(load().rtg_trace_nearest_instances_device(self.h, _ptr(d_rays), int(n), _ptr(d_hits),
                                                        _ptr(d_inst) if d_inst is not None else None, 0, stream))

    def trace_any_device(self, d_rays, n: int, d_occ, stream=None):
        check(load().rtg_trace_any_instances_device(self.h, _ptr(d_rays), int(n), _ptr(d_occ), 0, stream))

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and _lib is not None:
            _lib.rtg_instances_destroy(h)
            self.h = None


class Batch:
    """Scenes built together and traced together (rtg_batch_*).  `tasks` is a
    list of (scene_index, mode, d_rays, n, d_out) with device buffers (torch
    tensors or raw pointers)."""

    def __init__(self, scenes, ks, tasks):
        L = load()
        self._scenes = list(scenes)      # keep the scene objects alive
        self._keep = [t for t in tasks]
        arr = (C.c_void_p * len(scenes))(*[sc.h.value for sc in scenes])
        karr = (C.c_int32 * len(scenes))(*[int(k) for k in ks])
        tarr = (TraceTaskC * max(len(tasks), 1))()
        for i, (si, mode, rays, n, out) in enumerate(tasks):
            tarr[i] = TraceTaskC(int(si), int(mode), _ptr(rays), int(n), _ptr(out))
        h = C.c_void_p()
        check(L.rtg_batch_create(arr, len(scenes), karr, tarr, len(tasks), C.byref(h)))
        self.h = h

    def build_async(self, stream=None):
        check(load().rtg_batch_build_async(self.h, stream))

    def trace_async(self, stream=None):
        check(load().rtg_batch_trace_async(self.h, stream))

    def check(self, stream=None) -> int:
        return load().rtg_batch_check(self.h, stream)

    def rays(self) -> int:
        r = C.c_int64()
        check(load().rtg_batch_rays(self.h, C.byref(r)))
        return r.value

    def set_tuning(self, empty_run: int = None, persistent: bool = None, heavy_cell: int = None,
                   heavy_lanes: int = None, refill: int = None):
        if refill is not None:
            check(load().rtg_batch_set_tuning(self.h, RTG_TUNE_REFILL, int(refill)))
        if heavy_cell is not None:
            check(load().rtg_batch_set_tuning(self.h, RTG_TUNE_HEAVY_CELL, int(heavy_cell)))
        if heavy_lanes is not None:
            check(load().rtg_batch_set_tuning(self.h, RTG_TUNE_HEAVY_LANES, int(heavy_lanes)))
        if empty_run is not None:
            check(load().rtg_batch_set_tuning(self.h, RTG_TUNE_EMPTY_RUN, int(empty_run)))
        if persistent is not None:
            check(load().rtg_batch_set_tuning(self.h, RTG_TUNE_PERSISTENT, 1 if persistent else 0))

    def close(self):
        if getattr(self, "h", None):
            load().rtg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def serve(scenes, requests, pool_bytes: int, plain: bool = False, max_in_flight: int = 3,
          max_step_rays: int = 0, empty_run: int = 0):
    """Runs rtg_serve_run.  requests: list of (arrival_s, scene_index, mode,
    h_rays, n, h_out) with pinned host buffers (torch pinned tensors or
    pointers).  Returns (admit_s, done_s) arrays."""
    L = load()
    arr = (C.c_void_p * len(scenes))(*[sc.h.value for sc in scenes])
    reqs = (RequestC * max(len(requests), 1))()
    for i, (t, si, mode, rays, n, out) in enumerate(requests):
        reqs[i] = RequestC(float(t), int(si), int(mode), _ptr(rays), int(n), _ptr(out))
    times = (RequestTimesC * max(len(requests), 1))()
    opt = ServeOptionsC(int(pool_bytes), int(max_step_rays), int(max_in_flight), 1 if plain else 0, int(empty_run), 0)
    check(L.rtg_serve_run(arr, len(scenes), reqs, len(requests), C.byref(opt), times))
    admit = np.array([times[i].admit_s for i in range(len(requests))])
    done = np.array([times[i].done_s for i in range(len(requests))])
    return admit, done


def load_mesh(path: str):
    """-> (verts (V, 3) float32, tris (N, 3) int32, source_face (N,) int64,
    info dict) with the reference loaders' semantics (rtg_mesh_load)."""
    m = MeshC()
    check(load().rtg_mesh_load(str(path).encode(), C.byref(m)))
    try:
        verts = np.ctypeslib.as_array(m.verts, shape=(m.nverts * 3,)).reshape(-1, 3).copy() if m.nverts \
            else np.zeros((0, 3), np.float32)
        tris = np.ctypeslib.as_array(m.tris, shape=(m.ntris * 3,)).reshape(-1, 3).copy() if m.ntris \
            else np.zeros((0, 3), np.int32)
        face = np.ctypeslib.as_array(m.source_face, shape=(m.ntris,)).copy() if m.ntris else np.zeros(0, np.int64)
        info = dict(faces=int(m.faces), dropped=int(m.dropped))
    finally:
        load().rtg_mesh_free(C.byref(m))
    return verts, tris, face, info


def probe_read_gbs(device: int, nbytes: int, reps: int) -> float:
    """Read bandwidth over a buffer of nbytes (L2 when it fits, else HBM)."""
    out = C.c_double()
    check(load().rtg_probe_read_gbs(int(device), int(nbytes), int(reps), C.byref(out)))
    return out.value


def kernel_launches() -> int:
    return int(load().rtg_kernel_launch_count())


def split_hits(hits: np.ndarray) -> dict:
    hits = np.ascontiguousarray(hits).reshape(-1, 4)
    h32 = hits.view(np.float32) if hits.dtype != np.float32 else hits
    return dict(id=h32[:, 0].copy().view(np.int32), t=h32[:, 1].copy(), u=h32[:, 2].copy(), v=h32[:, 3].copy())
