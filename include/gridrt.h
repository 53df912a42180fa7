/*
 * gridrt.h -- C ABI of the GB300 uniform-grid ray tracer (libgridrt.so).
 *
 * Drop-in for the acceleration-structure path of potato3d/grid-rt:
 *   rt::IAccStructBuilder::buildGeometry(Geometry*)          include/rt/IAccStructBuilder.h:16
 *     implemented by rtp::UniformGridAccStructBuilder         src/rtplugins/UniformGridAccStructBuilder.cpp:58-149
 *   rt::IAccStruct::traceNearestGeometry(Instance, Ray&, Hit&) include/rt/IAccStruct.h:22
 *     implemented by rtp::UniformGridAccStruct               src/rtplugins/UniformGridAccStruct.cpp:30-42,113-196
 *   rt::IAccStruct::traceAnyGeometry(...)                    include/rt/IAccStruct.h:28 (a stub in the reference)
 * and of the CUDA tracer's host ABI (src/rtcuda/RayTracing.h:6-44), which this
 * replaces with handles, status codes and caller-owned host arrays.
 *
 * Conventions
 *  - Every call returns rtg_status.  Handles are opaque.  Host arrays stay
 *    owned by the caller; device buffers are owned by the library.
 *  - `stream` arguments are cudaStream_t passed as void*; NULL selects the
 *    scene's own stream.  Calls on one scene are ordered on that stream;
 *    trace calls on different streams may run concurrently once the scene is
 *    built (the grid is read-only during tracing, as the reference requires
 *    for its OpenMP renderers, src/rtplugins/MultiThreadRenderer.cpp:23-30).
 *  - Rays: 8 x float32 per ray {ox, oy, oz, tnear, dx, dy, dz, tfar}
 *    (rt::Ray orig/dir/tnear/tfar, include/rt/Ray.h:9-24).  The reference's
 *    trace entry initialises tnear = 2e-4 and tfar = FLT_MAX
 *    (src/rtcore/IAccStruct.cpp:33-36); callers that want that behaviour pass
 *    those values.
 *  - Hits: rtg_hit {id, t, u, v}; id = -1 for a miss.  u and v are the
 *    barycentric weights of vertices 1 and 2 (Hit::v1Coord / v2Coord,
 *    include/rt/Hit.h:9-17); the weight of vertex 0 is 1 - u - v.
 *  - Geometry: vertices float32 x 3, triangle indices int32 x 3 (rt::Geometry
 *    vertices + TriDesc::v, include/rt/Geometry.h:20-27).  Triangles must be
 *    valid in the sense of TriAccel::valid (src/rtcore/Triangle.cpp:57-63), as
 *    Context's PrimitiveBuilder guarantees before the builder runs.
 */
#ifndef GRIDRT_H
#define GRIDRT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes; the first three keep the values of RT_OK / RT_NO_MEMORY /
 * RT_INVALID_PARAM (include/rt/common.h:19-21). */
typedef enum {
    RTG_OK = 0,
    RTG_NO_MEMORY = 1,
    RTG_INVALID_PARAM = 3,
    RTG_DEVICE_ERROR = 4,
    RTG_TIMEOUT = 5,
    RTG_NOT_BUILT = 6,
    RTG_INVALID_GEOMETRY = 7
} rtg_status;

typedef struct rtg_scene_s* rtg_scene;

typedef struct {
    int32_t id;
    float t;
    float u;
    float v;
} rtg_hit;

/* Grid description, as UniformGridAccStruct stores it
 * (include/rtp/UniformGridAccStruct.h:49-56 plus IAccStruct::_bbox). */
typedef struct {
    int32_t res[3];
    float bmin[3];
    float bmax[3];
    float cell[3];
    float inv_cell[3];
    int64_t ncells;
    int64_t nrefs;
    int32_t k;
    int32_t built;
} rtg_grid_info;

/* Pinhole camera: the parameters of cudaSetCameraParameters
 * (src/rtcuda/RayTracing.h:20-23) plus the viewport.  Ray for pixel (x, y),
 * row 0 at the bottom: dir = base_dir + near_u*((x+0.5)/width) + near_v*((y+0.5)/height),
 * unnormalised (src/rtplugins/PinholeCamera.cpp:131-137). */
typedef struct {
    float eye[3];
    float base_dir[3];
    float near_u[3];
    float near_v[3];
    int32_t width;
    int32_t height;
    int32_t order;   /* RTG_ORDER_* : mapping of ray index -> pixel */
    int32_t pad;
} rtg_camera;

enum { RTG_ORDER_SCANLINE = 0, RTG_ORDER_MORTON8 = 1 };

/* Flags for trace calls. */
enum {
    RTG_TRACE_DEFAULT = 0,
    RTG_TRACE_COUNTERS = 1 /* accumulate cells visited / triangle tests (rtg_scene_counters) */
};

/* Library version and the device it runs on. */
const char* rtg_version(void);
/* Text of the last error on this thread. */
const char* rtg_last_error(void);

/* ---- scene lifetime ------------------------------------------------------
 * rtg_scene_create: device ordinal, optional stream (NULL: the library
 * creates a non-blocking stream for the scene).
 * Replaces rtInitContext (src/rtcuda/RayTracing.h:8). */
rtg_status rtg_scene_create(int device, void* stream, rtg_scene* out);
rtg_status rtg_scene_destroy(rtg_scene scene);
/* The stream that NULL selects for this scene. */
rtg_status rtg_scene_stream(rtg_scene scene, void** stream_out);

/* ---- geometry ------------------------------------------------------------
 * Copy vertices and triangles from HOST memory (cudaTransferTriangleVertices,
 * src/rtcuda/RayTracing.h:27).  Sizes may change between calls. */
rtg_status rtg_scene_set_geometry(rtg_scene scene, const float* verts, int64_t nverts, const int32_t* tris,
                                  int64_t ntris, void* stream);
/* Same, from DEVICE memory (no host round trip; the data is copied). */
rtg_status rtg_scene_set_geometry_device(rtg_scene scene, const float* d_verts, int64_t nverts,
                                         const int32_t* d_tris, int64_t ntris, void* stream);
/* Replace vertex positions only (same vertex count), host or device source. */
rtg_status rtg_scene_update_vertices(rtg_scene scene, const float* verts, int64_t nverts, int from_device,
                                     void* stream);
/* Displace every vertex along `normals` (float32 x 3 per vertex, device or
 * host) by amp*sin(freq*p.x + phase) from the base positions `base`
 * (device): the per-frame deformation of the deforming-mesh workload. */
rtg_status rtg_scene_deform_vertices(rtg_scene scene, const float* d_base, const float* d_normals, float amp,
                                     float freq, float phase, void* stream);

/* ---- grid build (UniformGridAccStructBuilder::buildGeometry) -------------
 * k = cells per triangle (the reference hard-codes 6,
 * src/rtplugins/UniformGridAccStructBuilder.cpp:91).  Synchronous: returns
 * after the grid is complete, growing device buffers as needed. */
rtg_status rtg_scene_build(rtg_scene scene, int32_t k, void* stream);
/* Asynchronous build for graph capture and pipelining: enqueues the build
 * using the current buffer capacities (the first build of a scene runs
 * synchronously to size them).  Trace calls may be enqueued right after it on
 * the same stream.  rtg_scene_build_check synchronises the stream and returns
 * RTG_OK, or RTG_NO_MEMORY when any build since the last check exceeded a
 * capacity (its traces returned misses; call rtg_scene_build). */
rtg_status rtg_scene_build_async(rtg_scene scene, int32_t k, void* stream);
rtg_status rtg_scene_build_check(rtg_scene scene, void* stream);
/* Reserve device capacity for grids of up to ncells cells and nrefs
 * (cell, triangle) references (avoids regrowth inside captured graphs). */
rtg_status rtg_scene_reserve(rtg_scene scene, int64_t ncells, int64_t nrefs);

rtg_status rtg_scene_grid_info(rtg_scene scene, rtg_grid_info* out);
/* Copy the CSR grid to host: offsets[ncells+1], ids[nrefs] (cell lists sorted
 * by triangle id, linear cell index x + y*nx + z*nx*ny). */
rtg_status rtg_scene_grid_download(rtg_scene scene, int32_t* offsets, int32_t* ids);
/* Copy the scene's current vertex positions to host (nverts x 3 float32),
 * e.g. after rtg_scene_deform_vertices. */
rtg_status rtg_scene_download_vertices(rtg_scene scene, float* verts);
/* Device pointers of the CSR grid and the triangle records (read-only use). */
rtg_status rtg_scene_grid_device(rtg_scene scene, const int32_t** d_offsets, const int32_t** d_ids,
                                 const float** d_tris);

/* ---- tracing -------------------------------------------------------------
 * Closest hit for n rays (UniformGridAccStruct::traceNearestGeometry).
 * rays / hits in HOST memory: the call copies in and out and synchronises. */
rtg_status rtg_trace_nearest(rtg_scene scene, const float* rays, int64_t n, rtg_hit* hits, int32_t flags,
                             void* stream);
/* rays / hits in DEVICE memory: asynchronous on `stream`. */
rtg_status rtg_trace_nearest_device(rtg_scene scene, const float* d_rays, int64_t n, rtg_hit* d_hits,
                                    int32_t flags, void* stream);
/* Shadow any-hit: occluded[i] = 1 iff the ray hits a triangle before its
 * tfar word (tmax).  HOST and DEVICE variants as above. */
rtg_status rtg_trace_any(rtg_scene scene, const float* rays, int64_t n, uint8_t* occluded, int32_t flags,
                         void* stream);
rtg_status rtg_trace_any_device(rtg_scene scene, const float* d_rays, int64_t n, uint8_t* d_occluded,
                                int32_t flags, void* stream);
/* Camera rays generated on the device (cudaRayTrace, src/rtcuda/RayTracing.h:42),
 * width*height closest hits into d_hits (ray i -> pixel per cam->order).
 * With d_shadow_rays != NULL a shadow ray toward the point light is also
 * written per pixel (SimplePointLight::illuminate, src/rtplugins/SimplePointLight.cpp:18-52;
 * Sample::initLightRay/initShadowRay, src/rtcore/Sample.cpp:22-42): origin
 * P + n*2e-4, direction light - origin (unnormalised), tnear 2e-4, tmax 1;
 * pixels without a shadow ray (miss, or surface facing away from the light)
 * get tmax = -1.  n is the flat normal turned to face the incoming ray. */
rtg_status rtg_trace_camera_device(rtg_scene scene, const rtg_camera* cam, rtg_hit* d_hits,
                                   const float* light_pos, float* d_shadow_rays, int32_t flags, void* stream);
/* Camera closest hits plus one cosine-weighted diffuse secondary ray per hit
 * (origin P + n*2e-4 with the flat normal n turned toward the incoming ray,
 * tnear 2e-4, tfar FLT_MAX; random bits from a counter-based hash of `seed`
 * and the ray index).  Pixels without a hit get a ray with tfar = -1, which
 * the trace calls report as a miss.  No counterpart in the reference's CPU
 * path; it feeds the skewed-density workload's secondary rays. */
rtg_status rtg_trace_camera_diffuse_device(rtg_scene scene, const rtg_camera* cam, uint64_t seed, rtg_hit* d_hits,
                                           float* d_secondary_rays, int32_t flags, void* stream);
/* Primary + shadow frame: camera closest hits and every hit's shadow ray
 * traced with the any-hit rules, the shadow ray in the same thread right
 * after its camera ray (one launch, plus the deferred-ray passes); the same
 * results as rtg_trace_camera_device followed by rtg_trace_any_device over
 * the shadow rays.  occluded[i]: 0 lit, 1 shadowed, 2 no shadow ray.
 * d_shadow_rays (optional, may be NULL: the scene's staging buffer is used)
 * receives the shadow rays as rtg_trace_camera_device writes them. */
rtg_status rtg_trace_frame_device(rtg_scene scene, const rtg_camera* cam, const float* light_pos,
                                  rtg_hit* d_hits, uint8_t* d_occluded, float* d_shadow_rays, void* stream);

/* The same frame with HOST outputs: copies hits (width*height rtg_hit) and
 * occluded (width*height bytes) back and synchronises. */
rtg_status rtg_trace_frame(rtg_scene scene, const rtg_camera* cam, const float* light_pos, rtg_hit* hits,
                           uint8_t* occluded, void* stream);

/* rtg_trace_frame for a frame loop, the frame-level render of
 * src/rtcuda/CudaRenderer.cpp:33-63 with its read-back overlapped: enqueues
 * the frame's two trace passes on `stream` and the copy of hits and
 * occlusion into the host buffers on a copy stream of the scene, and
 * returns without waiting; *ticket receives the frame's number (0, 1, ...).
 * The copy overlaps the next frames' builds and traces when the host
 * buffers are pinned (cudaMallocHost); with pageable buffers it is correct
 * but not overlapped.  Two frames' device outputs alternate: a frame's trace
 * waits, on the GPU, for the copy of the frame two before it.  The host
 * buffers are complete once rtg_trace_frame_wait(scene, ticket) returns and
 * must stay valid until then.  Enqueue a scene's frames on one stream. */
rtg_status rtg_trace_frame_async(rtg_scene scene, const rtg_camera* cam, const float* light_pos, rtg_hit* hits,
                                 uint8_t* occluded, void* stream, uint64_t* ticket);
/* Blocks until the frame with this ticket, and every frame before it, is in
 * its host buffers.  RTG_INVALID_PARAM for a ticket not yet issued. */
rtg_status rtg_trace_frame_wait(rtg_scene scene, uint64_t ticket);

/* Grid build that allocates no device memory.  It has no counterpart in the
 * reference; it exists for callers that must not let a library allocate GPU
 * memory: real-time frame loops, where an allocation and the synchronisation
 * it can bring would stall the frame, and applications that hand out every
 * byte of device memory from their own pool or allocator.
 * The caller passes device arrays: d_verts (nverts x 3 float32), d_tris
 * (ntris x 3 int32) and the outputs d_offsets (offsets_cap int32, 16-byte
 * aligned; the grid needs ncells + 1), d_ids (ids_cap int32; nrefs needed) and
 * d_tri_records (ntris x 12 float32, 16-byte aligned: v0|id, e1, e2).  The
 * result equals rtg_scene_build's grid bit for bit; *info receives the grid
 * description (also on RTG_NO_MEMORY, so the caller can size its buffers and
 * call again).  The build's working memory is one fixed device array inside
 * the library (about 3.2 MB on every GPU that loads the library, kept until
 * the process exits): at most 524,288 (cell, triangle) references and
 * 16,777,216 cells per call; larger grids return RTG_INVALID_PARAM.  The call
 * synchronises `stream` before returning.  All calls share that array: each
 * call clears what must start from zero, and calls that overlap on the GPU
 * (different streams or threads at once) race -- serialise them.  Every
 * call looks up the array's address (cudaGetSymbolAddress) on the device that
 * is current, so calls after a device reset use the new context's array; the
 * first call on a device also reads the device's limits -- make it before any
 * stream capture on that device. */
rtg_status rtg_grid_build_noalloc(const float* d_verts, int64_t nverts, const int32_t* d_tris, int64_t ntris,
                                  int32_t k, int32_t* d_offsets, int64_t offsets_cap, int32_t* d_ids,
                                  int64_t ids_cap, float* d_tri_records, rtg_grid_info* info, void* stream);

/* Number of CUDA kernels this library has launched in this process. */
uint64_t rtg_kernel_launch_count(void);

/* ---- batches: many scenes built and traced together ----------------------
 * A batch plan fixes a set of scenes (up to 64, same device, each non-empty)
 * and a set of trace tasks; its device tables are uploaded once, so the two
 * enqueue calls below can run every frame or be captured in a CUDA graph.
 *   rtg_batch_build_async: every scene's grid in one set of build kernels
 *     (block row y builds scene y); same result as rtg_scene_build per scene.
 *   rtg_batch_trace_async: every task in one persistent trace launch; warps
 *     claim 32-ray slices of the concatenated tasks.
 *   rtg_batch_check: synchronises and reports whether every build since the
 *     last check fitted its scene's buffers (RTG_NO_MEMORY otherwise: rebuild
 *     the scenes with rtg_scene_build and recreate the plan).
 * The enqueue calls re-upload a scene's table entry (synchronously) when its
 * buffers moved since the last call, e.g. after a growing rtg_scene_build; a
 * CUDA graph captured from them keeps the addresses it saw, so do not let the
 * scenes' buffers grow while such a graph is in use (rtg_scene_reserve). */
typedef struct rtg_batch_s* rtg_batch;
enum { RTG_MODE_NEAREST = 0, RTG_MODE_ANY = 1 };
typedef struct {
    int32_t scene;        /* index into the scenes array of rtg_batch_create */
    int32_t mode;         /* RTG_MODE_NEAREST (rtg_hit out) or RTG_MODE_ANY (uint8 out) */
    const float* d_rays;  /* n x 8 float32, device */
    int64_t n;
    void* d_out;          /* device output: n rtg_hit or n uint8 */
} rtg_trace_task;
/* k[i]: cells per triangle for scene i.  Scenes are built once here
 * (synchronously) to size their buffers. */
rtg_status rtg_batch_create(const rtg_scene* scenes, int32_t nscenes, const int32_t* k, const rtg_trace_task* tasks,
                            int32_t ntasks, rtg_batch* out);
rtg_status rtg_batch_build_async(rtg_batch batch, void* stream);
rtg_status rtg_batch_trace_async(rtg_batch batch, void* stream);
rtg_status rtg_batch_check(rtg_batch batch, void* stream);
/* Total rays over the batch's tasks. */
rtg_status rtg_batch_rays(rtg_batch batch, int64_t* rays);
/* Keys RTG_TUNE_EMPTY_RUN, RTG_TUNE_PERSISTENT, RTG_TUNE_HEAVY_CELL,
 * RTG_TUNE_HEAVY_LANES and RTG_TUNE_REFILL, as for rtg_scene_set_tuning (lane
 * refill stays within one task: a warp's rays share scene and mode);
 * cell-ordered records are a per-scene setting. */
rtg_status rtg_batch_set_tuning(rtg_batch batch, int32_t key, int32_t value);
rtg_status rtg_batch_destroy(rtg_batch batch);

/* ---- scene ingest ----------------------------------------------------------
 * rtg_mesh_load reads a .obj or .ply file into the arrays the grid build takes,
 * as the reference's rtdb loaders feed rt::PrimitiveBuilder
 * (src/rtdb/ObjFileLoader.cpp, src/rtdb/TriMeshLoader.cpp:17-84,
 * src/rtcore/PrimitiveBuilder.cpp): every face corner (OBJ) or triangle corner
 * (PLY) becomes a new vertex, polygons are split as fans (s, s+i, s+i+1), and
 * a triangle whose Wald record would hold an inf or NaN (TriAccel::valid,
 * src/rtcore/Triangle.cpp:55-63) is dropped with its successors renumbered, so
 * triangle ids are the reference's.  source_face[t] is the file face of
 * triangle t.  The arrays are the library's: release them with rtg_mesh_free. */
typedef struct {
    float* verts;          /* nverts x 3 */
    int64_t nverts;
    int32_t* tris;         /* ntris x 3 */
    int64_t ntris;
    int64_t* source_face;  /* ntris */
    int64_t faces;         /* faces read from the file */
    int64_t dropped;       /* triangles dropped as invalid */
} rtg_mesh;
rtg_status rtg_mesh_load(const char* path, rtg_mesh* out);
void rtg_mesh_free(rtg_mesh* mesh);
/* Loads a mesh file into the scene (rtg_scene_set_geometry); info (optional)
 * receives the counts and source_face (verts / tris set to NULL). */
rtg_status rtg_scene_load(rtg_scene scene, const char* path, rtg_mesh* info);

/* Animated keyframes, double-buffered: copies nverts x 3 floats from (pinned)
 * host memory into the scene's second vertex buffer on copy_stream -- after
 * the scene's last build, so it can overlap that frame's traces -- and the
 * scene's next build waits for the copy and builds from it (the buffers
 * swap).  The reference re-uploads each keyframe before its rebuild
 * (src/rtgl/GpuRenderer.cpp:97-129). */
rtg_status rtg_scene_stage_vertices(rtg_scene scene, const float* h_verts, int64_t nverts, void* copy_stream);

/* ---- shading wavefront ---------------------------------------------------
 * rtg_render renders a frame of one scene the way the reference's renderers
 * call Context::traceNearest per pixel and its materials shade the hit
 * (src/rtcore/Sample.cpp, src/rtplugins/{HeadlightMaterial,HeadlightMaterialColor,
 * PhongMaterial,PhongMaterialColor,SimplePointLight,SimpleEnvironment}.cpp), as
 * a wavefront: primary rays, then per recursion level one closest-hit trace of
 * every live ray, one any-hit trace of its shadow rays (one per point light),
 * one shading pass that spawns reflection / refraction rays, and finally the
 * per-pixel colours combined level by level in the reference's order
 * (local + reflexion * reflected + (1 - opacity) * refracted).
 * Shadow rays follow the GPU shader semantics (occluded when a hit lies
 * before the light); the reference's CPU any-hit is a stub.  Textures are
 * not applied.  Normals and colours are per vertex (RT_BIND_PER_VERTEX), the
 * material per triangle.  Synchronous: returns when d_rgb is written. */
enum {
    RTG_MAT_HEADLIGHT = 0,        /* vertex colours */
    RTG_MAT_HEADLIGHT_COLOR = 1,  /* material diffuse colour */
    RTG_MAT_PHONG = 2,            /* vertex colours */
    RTG_MAT_PHONG_COLOR = 3       /* material diffuse colour */
};
typedef struct {
    int32_t type;
    float ambient[3];
    float diffuse[3];
    float specular[3];
    float specular_exponent;
    float reflexion;              /* PhongMaterial::setReflexCoeff */
    float refraction_index;
    float opacity;
} rtg_material;
typedef struct {
    float position[3];
    float intensity[3];
    int32_t cast_shadows;
    int32_t pad;
} rtg_point_light;
typedef struct {
    const float* d_normals;       /* nverts x 3 (device) */
    const float* d_colors;        /* nverts x 3 (device), NULL: white */
    const int32_t* d_material;    /* ntris material indices (device), NULL: material 0 */
    const rtg_material* materials;   /* host */
    int32_t nmaterials;
    const rtg_point_light* lights;   /* host */
    int32_t nlights;
    float background[3];          /* SimpleEnvironment */
    int32_t max_depth;            /* Context::setMaxRecursionDepth (default 3) */
    float medium_index;           /* Context::setMediumRefractionIndex (default 1) */
} rtg_shading;
/* d_rgb: width x height x 3 float32, row-major from the bottom row (the
 * camera's pixel order, scanline).  rays_out (optional): rays traced in total
 * (primary, shadow, reflected, refracted). */
rtg_status rtg_render(rtg_scene scene, const rtg_camera* cam, const rtg_shading* shading, float* d_rgb,
                      int64_t* rays_out, void* stream);

/* ---- measurement ----------------------------------------------------------
 * Public diagnostic: the read bandwidth of this device over a buffer of
 * `bytes` (16-byte loads that bypass L1, `reps` passes, best of 5 timed
 * launches).  A buffer well inside L2 measures L2, one far above it HBM; a
 * caller uses it as the denominator of a trace's bandwidth fraction on the
 * machine at hand.  Allocates and frees the buffer; not for use while the
 * device runs other timed work. */
rtg_status rtg_probe_read_gbs(int32_t device, int64_t bytes, int32_t reps, double* gbs);

/* ---- two-level instancing -------------------------------------------------
 * The scene level of the reference's plugin interface: an ordered set of
 * instances, each a built scene placed by a 3 x 4 row-major matrix.
 *   rtg_instances_create   Context::instantiateGeometry for every instance +
 *                          IAccStructBuilder::buildInstance (src/rtcore/Context.cpp:352-390,
 *                          src/rtcore/IAccStructBuilder.cpp:16-33): world box of each
 *                          instance (its grid box's corners transformed, 1% enlarged) and
 *                          the scene box over all of them
 *   rtg_trace_nearest_instances*  IAccStruct::traceNearestInstance
 *                          (src/rtcore/IAccStruct.cpp:26-72): the ray is clipped against the
 *                          scene box, then taken to each instance's local space in order
 *                          (origin by local_from_world, direction by its 3 x 3 part, not
 *                          renormalised) and traced from the best distance so far, so a
 *                          later instance wins only with a strictly closer hit
 *   rtg_trace_any_instances_device  occlusion: closest hit over all instances before
 *                          the ray's tfar word (the reference's any-hit is a stub)
 * Rows are applied as x' = ((m0 x + m1 y) + m2 z) + m3, one float rounding per
 * operation.  The instance boxes are taken at create / update: call
 * rtg_instances_update after rebuilding a member scene.  d_instance receives
 * the winning instance's index (-1 on a miss); t is the same in world and
 * local space, u / v are barycentrics of the local triangle. */
typedef struct rtg_instances_s* rtg_instances;
typedef struct {
    rtg_scene scene;              /* built scene */
    float world_from_local[12];   /* 3 x 4 row-major */
    float local_from_world[12];   /* its inverse, applied to rays */
} rtg_instance;
rtg_status rtg_instances_create(const rtg_instance* inst, int32_t n, rtg_instances* out);
rtg_status rtg_instances_update(rtg_instances set, const rtg_instance* inst, int32_t n);
/* box: scene box {min xyz, max xyz}; inst_boxes (optional): 6 floats per instance. */
rtg_status rtg_instances_box(rtg_instances set, float box[6], float* inst_boxes);
/* Keys RTG_TUNE_EMPTY_RUN (2, 4, 8) and RTG_TUNE_PERSISTENT. */
rtg_status rtg_instances_set_tuning(rtg_instances set, int32_t key, int32_t value);
rtg_status rtg_trace_nearest_instances_device(rtg_instances set, const float* d_rays, int64_t n, rtg_hit* d_hits,
                                              int32_t* d_instance, int32_t flags, void* stream);
rtg_status rtg_trace_any_instances_device(rtg_instances set, const float* d_rays, int64_t n, uint8_t* d_occ,
                                          int32_t flags, void* stream);
/* Host arrays; instance (optional) receives the winning instance per ray. */
rtg_status rtg_trace_nearest_instances(rtg_instances set, const float* rays, int64_t n, rtg_hit* hits,
                                       int32_t* instance, void* stream);
rtg_status rtg_instances_destroy(rtg_instances set);

/* ---- serving: continuous batching over resident scenes ------------------
 * rtg_serve_run replays a stream of ray-query requests in real time against
 * built, resident scenes (up to 64, one device) and reports, per request, when
 * it was admitted and when its results were back in host memory.  Requests
 * are admitted in arrival order while a device pool of opt->pool_bytes has
 * room for their rays (32 B/ray) and results (16 B or 1 B per ray); the
 * admitted requests form one step: uploads, ONE persistent trace launch over
 * all of them, downloads, on the step's own stream, up to opt->max_in_flight
 * steps on the GPU at once.  opt->plain = 1 instead serves one request at a
 * time through the single-scene trace (the per-request baseline).
 * h_rays / h_out must be pinned host memory; arrivals must be sorted. */
typedef struct {
    double arrival_s;     /* seconds after the start of the run */
    int32_t scene;        /* index into the scenes array */
    int32_t mode;         /* RTG_MODE_NEAREST or RTG_MODE_ANY (occlusion before each ray's tfar) */
    const float* h_rays;  /* n x 8 float32, pinned host */
    int64_t n;
    void* h_out;          /* n rtg_hit or n uint8 (0 lit, 1 occluded, 2 no ray), pinned host */
} rtg_request;
typedef struct {
    double admit_s;       /* its step was launched */
    double done_s;        /* its results were back in host memory */
} rtg_request_times;
typedef struct {
    int64_t pool_bytes;       /* device memory for requests in flight */
    int64_t max_step_rays;    /* rays per step at most (0: 16M) */
    int32_t max_in_flight;    /* steps on the GPU at once, 1..8 */
    int32_t plain;            /* 1: one request at a time, single-scene trace */
    int32_t empty_run;        /* trace tuning, 0 = the first scene's */
    int32_t pad;
} rtg_serve_options;
rtg_status rtg_serve_run(const rtg_scene* scenes, int32_t nscenes, const rtg_request* reqs, int64_t nreq,
                         const rtg_serve_options* opt, rtg_request_times* times);

/* Trace launch shape for this scene (results never depend on it):
 *   RTG_TUNE_EMPTY_RUN   empty cells a ray may walk per loop turn: 2, 4, 8, 16 (default 4)
 *   RTG_TUNE_PERSISTENT  1: persistent warps claim ray batches (default); 0: one batch per warp.
 *                        A persistent launch holds every SM's slots until it ends; a one-shot
 *                        launch's blocks retire as they finish, so traces of two scenes in
 *                        flight on their own streams share the SMs (1024^2 frames two in
 *                        flight: 3,846 Mrays/s persistent, 4,392 one-shot with blocks of 64;
 *                        one frame at a time persistent is the faster, ~3,470 against 3,367)
 *   RTG_TUNE_CELL_RECORDS 1: builds also store the triangle records in cell-list order
 *                        (48 B per reference) so traces skip the id indirection; from the next build
 *   RTG_TUNE_HEAVY_CELL  n > 0: a ray that meets a cell list longer than n is finished by a
 *                        second pass that traces it with a group of lanes (the list split
 *                        over them); default 32, 0 off.  Results are identical either way.
 *                        A ray that then meets a list above 2,048 entries (a dense cluster)
 *                        is finished by a third pass, one block of threads per ray, when the
 *                        scene's last checked build had such a list.
 *                        Costs 19 MB of device memory per scene (the passes' ray queues).
 *   RTG_TUNE_HEAVY_LANES lanes that trace one deferred ray together: 4, 8, 16, 32 (default)
 *   RTG_TUNE_REFILL      n in 1..32: a warp hands new rays to its idle lanes whenever at least
 *                        n are idle, instead of finishing each batch of 32 rays first (pays on
 *                        incoherent rays: +50 to +65% on random in-box rays at 16; 8 gains a
 *                        little more there and costs ~5% on camera rays); 0 off.  Unset, it is
 *                        16 for rays given as arrays (nearest, any, batches) and off for camera
 *                        and frame traces, whose lanes follow a camera ray with its shadow ray
 *   RTG_TUNE_BLOCK       threads per block of the one-lane trace launch: 64, 128 (default) or 256
 *                        (every block size keeps 64 registers a thread and 32 warps an SM)
 *   RTG_TUNE_LANES       lanes that trace each ray from its start: 1 (default: one ray a lane,
 *                        the long lists handed on as above), 2 or 4 (every ray walked by a group
 *                        of lanes that splits each cell's list).  Groups pay on launches too
 *                        small to fill the GPU with one ray a lane (65,536 triangles, 512^2
 *                        camera rays + their shadow rays: +41% at 2) and cost on full ones
 *                        (1024^2 frames: -44% at 2) */
enum {
    RTG_TUNE_EMPTY_RUN = 1,
    RTG_TUNE_PERSISTENT = 2,
    RTG_TUNE_CELL_RECORDS = 3,
    RTG_TUNE_HEAVY_CELL = 4,
    RTG_TUNE_HEAVY_LANES = 5,
    RTG_TUNE_REFILL = 6,
    RTG_TUNE_BLOCK = 7,
    RTG_TUNE_LANES = 8
};
rtg_status rtg_scene_set_tuning(rtg_scene scene, int32_t key, int32_t value);

/* Counters accumulated by calls made with RTG_TRACE_COUNTERS since the last
 * reset: out[0] = rays, out[1] = cells visited, out[2] = triangle tests. */
rtg_status rtg_scene_counters(rtg_scene scene, int64_t out[3], int reset);

#ifdef __cplusplus
}
#endif
#endif
