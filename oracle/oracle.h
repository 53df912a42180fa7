/*
 * oracle.h -- CPU restatement of the reference's uniform-grid build and
 * 3D-DDA trace (potato3d/grid-rt).  TEST INFRASTRUCTURE ONLY: tests, the
 * smoke check and bench.py's CPU-baseline leg may load liboracle.so; the
 * product (libgridrt.so) never links or calls it.
 *
 * Parity of this restatement is pinned against the reference's own sources
 * compiled unmodified (oracle/_ref, built by `make ref` where the reference
 * checkout exists) on seeded scenes, and against the committed golden
 * fixtures in tests/golden/ that were produced by that compiled reference.
 *
 * Array conventions (all little-endian, row-major):
 *   verts  : nverts x 3 float32
 *   idx    : ntris  x 3 int32
 *   rays   : n x 8 float32 {ox, oy, oz, tnear, dx, dy, dz, tfar}
 *   hits   : n x 4 32-bit words {id (int32, -1 = miss), t, u, v}
 *            u = Hit::v1Coord, v = Hit::v2Coord (src/rtcore/RayTriIntersection.cpp:43-47)
 *   grid CSR: offsets[ncells + 1] int32, ids[nrefs] int32, linear cell index
 *            x + y*nx + z*nx*ny (src/rtplugins/UniformGridAccStruct.cpp:82-90)
 */
#ifndef GRIDRT_ORACLE_H
#define GRIDRT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int32_t res[3];     /* nx, ny, nz */
    float bmin[3];      /* grid box (scene box enlarged by 1%) */
    float bmax[3];
    float cell[3];      /* cell size */
    float inv_cell[3];  /* 1 / cell size */
    int64_t ncells;
    int64_t nrefs;
} orc_grid_info;

/* Scene box, 1% enlargement and resolution rule with cells-per-triangle k.
 * Returns 0 on success, nonzero for empty input. */
int orc_grid_params(const float* verts, int64_t nverts, int64_t ntris, int32_t k, orc_grid_info* out);

/* Full CSR build.  Call once with offsets == ids == NULL to obtain info
 * (ncells, nrefs), then again with arrays of ncells+1 and nrefs entries. */
int orc_grid_build(const float* verts, int64_t nverts, const int32_t* idx, int64_t ntris, int32_t k,
                   orc_grid_info* info, int32_t* offsets, int32_t* ids);

/* Wald projection records, 12 words per triangle (rt::TriAccel layout). */
void orc_triaccel_build(const float* verts, const int32_t* idx, int64_t ntris, float* acc);

/* Closest hit through the grid.  counters (optional) receives 2 int64 per
 * ray: cells visited and triangle tests.  nthreads <= 0 uses all cores. */
void orc_trace_closest(const orc_grid_info* g, const int32_t* offsets, const int32_t* ids, const float* acc,
                       const float* rays, int64_t n, float* hits, int64_t* counters, int nthreads);

/* Shadow any-hit: occluded[i] = 1 iff the closest hit (tnear, tfar = tmax)
 * exists with t < tmax, where tmax is the ray's tfar word. */
void orc_trace_any(const orc_grid_info* g, const int32_t* offsets, const int32_t* ids, const float* acc,
                   const float* rays, int64_t n, uint8_t* occluded, int64_t* counters, int nthreads);

/* Moller-Trumbore in double for (ray i, triangle tri[i]); out: n x 3 {t, u, v}
 * (NaN where tri[i] < 0). */
void orc_mt_f64(const float* verts, const int32_t* idx, const float* rays, const int32_t* tri, int64_t n,
                double* out);

/* Two-level instancing (see oracle.c): xf / inv are 3 x 4 row-major
 * world_from_local / local_from_world matrices.  orc_instance_box gives an
 * instance's world box from its geometry's grid box, orc_scene_box the union
 * of ninst instance boxes (6 floats each: min xyz, max xyz). */
void orc_instance_box(const float* gbmin, const float* gbmax, const float* xf, float* bmin, float* bmax);
void orc_scene_box(int32_t ninst, const float* inst_boxes, float* box);
/* hits (n x 4 words) / inst_out (instance index, -1 = miss) / occluded may be
 * NULL independently. */
void orc_trace_instances(int32_t ninst, const orc_grid_info* const* g, const int32_t* const* offsets,
                         const int32_t* const* ids, const float* const* acc, const float* inv, const float* box,
                         const float* rays, int64_t n, float* hits, int32_t* inst_out, uint8_t* occluded,
                         int nthreads);

/* Shading (see oracle.c): materials and point lights with the layout of the
 * library's rtg_material / rtg_point_light; primary rays n x 8; rgb n x 3.
 * Returns the rays traced (primary, shadow, reflected, refracted). */
typedef struct {
    int32_t type;   /* 0 headlight, 1 headlight colour, 2 phong, 3 phong colour */
    float ambient[3], diffuse[3], specular[3];
    float specular_exponent, reflexion, refraction_index, opacity;
} orc_material;
typedef struct {
    float position[3], intensity[3];
    int32_t cast_shadows, pad;
} orc_light;
int64_t orc_render(const orc_grid_info* g, const int32_t* offsets, const int32_t* ids, const float* acc,
                   const int32_t* idx, const float* normals, const float* colors, const int32_t* material,
                   const orc_material* mats, int32_t nmats, const orc_light* lights, int32_t nlights,
                   const float* background, int32_t max_depth, float medium, const float* primary, int64_t n,
                   float* rgb, int nthreads);

/* Number of OpenMP threads the trace entry points use when nthreads <= 0. */
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
