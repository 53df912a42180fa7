/*
 * oracle.c -- CPU restatement of the reference's uniform-grid path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Every function below states the
 * reference lines it follows (paths relative to the reference project).  The
 * arithmetic is written operation by operation in the same order as the
 * reference, in float, and must be compiled without FMA contraction
 * (-ffp-contract=off) so x86-64 and aarch64 give identical bits.
 *
 * Semantics of the external `vr` helpers are the ones fixed in
 * oracle/shim/vr/common.h (sign, signBit, min, max, abs, MAX_VALUE).
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- vr helpers (shim semantics) -------------------------------------- */
static inline float vmin(float a, float b) { return a < b ? a : b; }
static inline float vmax(float a, float b) { return a > b ? a : b; }
static inline float vabs(float x) { return x < 0.0f ? -x : x; }
static inline int32_t vclamp(int32_t v, int32_t lo, int32_t hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline int32_t vsign(float x) { return x < 0.0f ? -1 : (x > 0.0f ? 1 : 0); }
static inline int32_t vsignbit(float x) { return signbit(x) ? 1 : 0; }

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---- a1/a2: scene box, 1% enlargement, resolution ---------------------
 * Aabb::buildFrom / expandBy      src/rtcore/Aabb.cpp:11-53
 * Aabb::scaleBy(0.01f, 0.01f)     src/rtcore/Aabb.cpp:78-91
 * resolution rule                 src/rtplugins/UniformGridAccStructBuilder.cpp:73-102
 * UniformGridAccStruct::setResolution src/rtplugins/UniformGridAccStruct.cpp:44-63 */
int orc_grid_params(const float* verts, int64_t nverts, int64_t ntris, int32_t k, orc_grid_info* out) {
    memset(out, 0, sizeof(*out));
    if (nverts <= 0 || ntris <= 0) return 1;
    float mn[3], mx[3];
    for (int d = 0; d < 3; ++d) mn[d] = mx[d] = verts[d];
    for (int64_t i = 1; i < nverts; ++i) {
        for (int d = 0; d < 3; ++d) {
            float v = verts[3 * i + d];
            if (v < mn[d])
                mn[d] = v;
            else if (v > mx[d])
                mx[d] = v;
        }
    }
    for (int d = 0; d < 3; ++d) {
        float s;
        if (mn[d] == mx[d])
            s = 0.01f;
        else
            s = vabs(mx[d] - mn[d]) * 0.01f;
        mn[d] -= s;
        mx[d] += s;
    }
    float diag[3];
    for (int d = 0; d < 3; ++d) diag[d] = mx[d] - mn[d];
    float V = diag[0] * diag[1] * diag[2];
    int32_t tri_count = (int32_t)ntris;
    float factor = powf((float)(k * tri_count) / V, 1.0f / 3.0f);
    for (int d = 0; d < 3; ++d) out->res[d] = (int32_t)ceilf(diag[d] * factor);
    for (int d = 0; d < 3; ++d) {
        out->bmin[d] = mn[d];
        out->bmax[d] = mx[d];
        out->cell[d] = (mx[d] - mn[d]) / (float)out->res[d];
        out->inv_cell[d] = 1.0f / out->cell[d];
    }
    out->ncells = (int64_t)out->res[0] * out->res[1] * out->res[2];
    return 0;
}

/* UniformGridAccStruct::worldToVoxel  src/rtplugins/UniformGridAccStruct.cpp:92-98 */
static inline int32_t world_to_voxel(const orc_grid_info* g, float v, int axis) {
    float t = (float)(v - g->bmin[axis]);
    float s = (float)(t * g->inv_cell[axis]);
    return (int32_t)s;
}

/* UniformGridAccStruct::voxelToWorld  src/rtplugins/UniformGridAccStruct.cpp:100-103 */
static inline float voxel_to_world(const orc_grid_info* g, int32_t vox, int axis) {
    float a = (float)vox * g->cell[axis];
    return a + g->bmin[axis];
}

/* Per-triangle cell range  src/rtplugins/UniformGridAccStructBuilder.cpp:111-127 */
static void tri_range(const orc_grid_info* g, const float* verts, const int32_t* idx, int64_t t, int32_t lo[3],
                      int32_t hi[3]) {
    const float* v0 = verts + 3 * (int64_t)idx[3 * t + 0];
    const float* v1 = verts + 3 * (int64_t)idx[3 * t + 1];
    const float* v2 = verts + 3 * (int64_t)idx[3 * t + 2];
    float bmn[3], bmx[3];
    for (int d = 0; d < 3; ++d) bmn[d] = bmx[d] = v0[d];
    for (int d = 0; d < 3; ++d) {
        if (v1[d] < bmn[d])
            bmn[d] = v1[d];
        else if (v1[d] > bmx[d])
            bmx[d] = v1[d];
    }
    for (int d = 0; d < 3; ++d) {
        if (v2[d] < bmn[d])
            bmn[d] = v2[d];
        else if (v2[d] > bmx[d])
            bmx[d] = v2[d];
    }
    for (int d = 0; d < 3; ++d) {
        lo[d] = world_to_voxel(g, bmn[d], d);
        hi[d] = world_to_voxel(g, bmx[d], d);
    }
}

/* ---- a3/a4: cell insertion in triangle order --------------------------
 * src/rtplugins/UniformGridAccStructBuilder.cpp:109-145 (the triangle/box
 * overlap test at :140 is commented out in the reference, so every cell of
 * the triangle's box range receives the triangle).  Lists come out sorted by
 * triangle id because triangles are appended in id order. */
int orc_grid_build(const float* verts, int64_t nverts, const int32_t* idx, int64_t ntris, int32_t k,
                   orc_grid_info* info, int32_t* offsets, int32_t* ids) {
    if (orc_grid_params(verts, nverts, ntris, k, info)) return 1;
    const int32_t nx = info->res[0], ny = info->res[1];
    int64_t C = info->ncells;
    int64_t* cnt = (int64_t*)calloc((size_t)C + 1, sizeof(int64_t));
    if (!cnt) return 2;
    int64_t R = 0;
    for (int64_t t = 0; t < ntris; ++t) {
        int32_t lo[3], hi[3];
        tri_range(info, verts, idx, t, lo, hi);
        for (int32_t z = lo[2]; z <= hi[2]; ++z)
            for (int32_t y = lo[1]; y <= hi[1]; ++y)
                for (int32_t x = lo[0]; x <= hi[0]; ++x) {
                    cnt[(int64_t)x + (int64_t)y * nx + (int64_t)z * nx * ny]++;
                    ++R;
                }
    }
    info->nrefs = R;
    if (!offsets || !ids) {
        free(cnt);
        return 0;
    }
    int64_t run = 0;
    for (int64_t c = 0; c < C; ++c) {
        int64_t n = cnt[c];
        offsets[c] = (int32_t)run;
        cnt[c] = run;
        run += n;
    }
    offsets[C] = (int32_t)run;
    for (int64_t t = 0; t < ntris; ++t) {
        int32_t lo[3], hi[3];
        tri_range(info, verts, idx, t, lo, hi);
        for (int32_t z = lo[2]; z <= hi[2]; ++z)
            for (int32_t y = lo[1]; y <= hi[1]; ++y)
                for (int32_t x = lo[0]; x <= hi[0]; ++x)
                    ids[cnt[(int64_t)x + (int64_t)y * nx + (int64_t)z * nx * ny]++] = (int32_t)t;
    }
    free(cnt);
    return 0;
}

/* ---- a6: Wald projection record --------------------------------------
 * TriAccel::buildFrom  src/rtcore/Triangle.cpp:11-55 */
void orc_triaccel_build(const float* verts, const int32_t* idx, int64_t ntris, float* acc) {
    for (int64_t t = 0; t < ntris; ++t) {
        const float* v0 = verts + 3 * (int64_t)idx[3 * t + 0];
        const float* v1 = verts + 3 * (int64_t)idx[3 * t + 1];
        const float* v2 = verts + 3 * (int64_t)idx[3 * t + 2];
        float b[3], c[3], n[3];
        for (int d = 0; d < 3; ++d) {
            b[d] = v2[d] - v0[d];
            c[d] = v1[d] - v0[d];
        }
        /* normal = c x b */
        n[0] = c[1] * b[2] - c[2] * b[1];
        n[1] = c[2] * b[0] - c[0] * b[2];
        n[2] = c[0] * b[1] - c[1] * b[0];
        uint32_t kk;
        if ((vabs(n[0]) > vabs(n[1])) && (vabs(n[0]) > vabs(n[2])))
            kk = 0;
        else if (vabs(n[1]) > vabs(n[2]))
            kk = 1;
        else
            kk = 2;
        uint32_t u = (kk + 1) % 3, v = (kk + 2) % 3;
        float* a = acc + 12 * t;
        uint32_t kw = kk;
        memcpy(&a[0], &kw, 4);
        a[1] = n[u] / n[kk];
        a[2] = n[v] / n[kk];
        float inv_nk = 1.0f / n[kk];
        float nl[3] = {n[0] * inv_nk, n[1] * inv_nk, n[2] * inv_nk};
        a[3] = v0[0] * nl[0] + v0[1] * nl[1] + v0[2] * nl[2];
        float inv_den = 1.0f / (b[u] * c[v] - b[v] * c[u]);
        a[4] = -b[v] * inv_den;
        a[5] = b[u] * inv_den;
        a[6] = (b[v] * v0[u] - b[u] * v0[v]) * inv_den;
        a[7] = 0.0f;
        a[8] = c[v] * inv_den;
        a[9] = -c[u] * inv_den;
        a[10] = (c[u] * v0[v] - c[v] * v0[u]) * inv_den;
        uint32_t tid = (uint32_t)t;
        memcpy(&a[11], &tid, 4);
    }
}

/* ---- a7..a9: ray setup, box clip, 3D-DDA, Wald test -------------------- */
typedef struct {
    float orig[3], dir[3], inv[3];
    float tnear, tfar;
    int32_t sgn[3], sbit[3];
} oray;

/* Ray::update  include/rt/Ray.h:26-37 */
static inline void ray_update(oray* r) {
    for (int d = 0; d < 3; ++d) {
        r->inv[d] = 1.0f / r->dir[d];
        r->sgn[d] = vsign(r->dir[d]);
        r->sbit[d] = vsignbit(r->dir[d]);
    }
}

/* AabbIntersection::clipRay  src/rtcore/AabbIntersection.cpp:37-63 */
static inline int clip_ray(const orc_grid_info* g, oray* r) {
    float rn = r->tnear, rf = r->tfar;
    for (int i = 0; i < 3; ++i) {
        float tn = (g->bmin[i] - r->orig[i]) * r->inv[i];
        float tf = (g->bmax[i] - r->orig[i]) * r->inv[i];
        rn = vmax(rn, vmin(tn, tf));
        rf = vmin(rf, vmax(tn, tf));
    }
    if (rn > rf) return 0;
    r->tnear = rn;
    r->tfar = rf;
    return 1;
}

static const uint32_t s_modulo[8] = {0, 1, 2, 0, 1, 2, 0, 1};
#define HIT_EPSILON 1e-4f

typedef struct {
    int32_t id;
    float u, v;
} ohit;

/* RayTriIntersection::hitWald  src/rtcore/RayTriIntersection.cpp:12-48 */
static inline void hit_wald(const float* a, const oray* r, ohit* h, float* best) {
    uint32_t k;
    memcpy(&k, &a[0], 4);
    const uint32_t ku = s_modulo[k + 1], kv = s_modulo[k + 2];
    const float nd = 1.0f / (r->dir[k] + a[1] * r->dir[ku] + a[2] * r->dir[kv]);
    const float f = nd * (a[3] - r->orig[k] - a[1] * r->orig[ku] - a[2] * r->orig[kv]);
    if ((f >= *best) || (f < r->tnear - HIT_EPSILON) || (f > r->tfar + HIT_EPSILON)) return;
    const float hu = r->orig[ku] + f * r->dir[ku];
    const float hv = r->orig[kv] + f * r->dir[kv];
    const float lambda = hu * a[4] + hv * a[5] + a[6];
    if (lambda < 0.0f) return;
    const float mue = hu * a[8] + hv * a[9] + a[10];
    if (mue < 0.0f) return;
    const float psi = 1.0f - lambda - mue;
    if (psi < 0.0f) return;
    *best = f;
    uint32_t tid;
    memcpy(&tid, &a[11], 4);
    h->id = (int32_t)tid;
    h->u = lambda;
    h->v = mue;
}

/* UniformGridAccStruct::traceNearestGeometry + traverse3ddda + intersectTriangles
 * src/rtplugins/UniformGridAccStruct.cpp:30-42, 113-196, 362-378.
 * Returns 1 with *t_out / *h on a hit.  cells/tests count the loop iterations
 * and Wald tests (for the algorithmic-bytes figure). */
static int trace_one_from(const orc_grid_info* g, const int32_t* offsets, const int32_t* ids, const float* acc,
                          oray* r, ohit* h, float* t_out, int64_t* cells, int64_t* tests, float hit_distance);

static int trace_one(const orc_grid_info* g, const int32_t* offsets, const int32_t* ids, const float* acc, oray* r,
                     ohit* h, float* t_out, int64_t* cells, int64_t* tests) {
    return trace_one_from(g, offsets, ids, acc, r, h, t_out, cells, tests, FLT_MAX);
}

/* hit_distance: the caller's best so far (Hit::distance on entry, which the
 * reference carries from one instance to the next). */
static int trace_one_from(const orc_grid_info* g, const int32_t* offsets, const int32_t* ids, const float* acc,
                          oray* r, ohit* h, float* t_out, int64_t* cells, int64_t* tests, float hit_distance) {
    if (!clip_ray(g, r)) return 0;
    const int32_t nx = g->res[0], ny = g->res[1], nz = g->res[2];
    float sp[3];
    for (int d = 0; d < 3; ++d) {
        float m = r->dir[d] * r->tnear;
        sp[d] = r->orig[d] + m;
    }
    int32_t x = vclamp(world_to_voxel(g, sp[0], 0), 0, nx - 1);
    int32_t y = vclamp(world_to_voxel(g, sp[1], 1), 0, ny - 1);
    int32_t z = vclamp(world_to_voxel(g, sp[2], 2), 0, nz - 1);
    const int32_t stepX = r->sgn[0], stepY = r->sgn[1], stepZ = r->sgn[2];
    const int32_t outX = -r->sbit[0] + nx * !r->sbit[0];
    const int32_t outY = -r->sbit[1] + ny * !r->sbit[1];
    const int32_t outZ = -r->sbit[2] + nz * !r->sbit[2];
    const float tDeltaX = vabs(g->cell[0] * r->inv[0]);
    const float tDeltaY = vabs(g->cell[1] * r->inv[1]);
    const float tDeltaZ = vabs(g->cell[2] * r->inv[2]);
    float tMaxX = (voxel_to_world(g, x + !r->sbit[0], 0) - r->orig[0]) * r->inv[0];
    float tMaxY = (voxel_to_world(g, y + !r->sbit[1], 1) - r->orig[1]) * r->inv[1];
    float tMaxZ = (voxel_to_world(g, z + !r->sbit[2], 2) - r->orig[2]) * r->inv[2];
    float best = hit_distance;
    do {
        const int64_t c = (int64_t)x + (int64_t)y * nx + (int64_t)z * nx * ny;
        const int32_t b = offsets[c], e = offsets[c + 1];
        if (cells) ++*cells;
        if (b != e) {
            r->tfar = vmin(vmin(tMaxX, tMaxY), tMaxZ);
            for (int32_t i = b; i < e; ++i) hit_wald(acc + 12 * (int64_t)ids[i], r, h, &best);
            if (tests) *tests += (e - b);
            if (best < hit_distance) {
                *t_out = best;
                return 1;
            }
        }
        if (tMaxX < tMaxY && tMaxX < tMaxZ) {
            x += stepX;
            tMaxX += tDeltaX;
        } else if (tMaxY < tMaxZ) {
            y += stepY;
            tMaxY += tDeltaY;
        } else {
            z += stepZ;
            tMaxZ += tDeltaZ;
        }
    } while (x != outX && y != outY && z != outZ);
    return 0;
}

static inline void load_ray(const float* q, oray* r) {
    r->orig[0] = q[0]; r->orig[1] = q[1]; r->orig[2] = q[2];
    r->tnear = q[3];
    r->dir[0] = q[4]; r->dir[1] = q[5]; r->dir[2] = q[6];
    r->tfar = q[7];
    ray_update(r);
}

void orc_trace_closest(const orc_grid_info* g, const int32_t* offsets, const int32_t* ids, const float* acc,
                       const float* rays, int64_t n, float* hits, int64_t* counters, int nthreads) {
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
#endif
    for (int64_t i = 0; i < n; ++i) {
        oray r;
        load_ray(rays + 8 * i, &r);
        ohit h = {-1, 0.f, 0.f};
        float t = 0.f;
        int64_t cells = 0, tests = 0;
        int found = (g->ncells > 0) && trace_one(g, offsets, ids, acc, &r, &h, &t, &cells, &tests);
        int32_t id = found ? h.id : -1;
        float* o = hits + 4 * i;
        memcpy(&o[0], &id, 4);
        o[1] = found ? t : 0.f;
        o[2] = found ? h.u : 0.f;
        o[3] = found ? h.v : 0.f;
        if (counters) {
            counters[2 * i] = cells;
            counters[2 * i + 1] = tests;
        }
    }
}

/* Shadow any-hit.  The reference's CPU any-hit entry points are stubs that
 * return false (src/rtcore/IAccStruct.cpp:108-122), so occlusion is defined
 * from the closest-hit traversal: occluded iff the first cell with an accepted
 * hit yields t < tmax.  GPU semantics cited: findAnyHit in
 * shaders/shadow_FRAG.glsl:147-245. */
void orc_trace_any(const orc_grid_info* g, const int32_t* offsets, const int32_t* ids, const float* acc,
                   const float* rays, int64_t n, uint8_t* occluded, int64_t* counters, int nthreads) {
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
#endif
    for (int64_t i = 0; i < n; ++i) {
        oray r;
        load_ray(rays + 8 * i, &r);
        const float tmax = rays[8 * i + 7];
        ohit h = {-1, 0.f, 0.f};
        float t = 0.f;
        int64_t cells = 0, tests = 0;
        int found = (g->ncells > 0) && trace_one(g, offsets, ids, acc, &r, &h, &t, &cells, &tests);
        occluded[i] = (uint8_t)(found && t < tmax);
        if (counters) {
            counters[2 * i] = cells;
            counters[2 * i + 1] = tests;
        }
    }
}

/* Moller-Trumbore in double (the published algorithm, Moller & Trumbore 1997;
 * float form in the reference at src/rtcore/RayTriIntersection.cpp:50-100). */
void orc_mt_f64(const float* verts, const int32_t* idx, const float* rays, const int32_t* tri, int64_t n,
                double* out) {
    for (int64_t i = 0; i < n; ++i) {
        double* o = out + 3 * i;
        if (tri[i] < 0) {
            o[0] = o[1] = o[2] = NAN;
            continue;
        }
        const float* q = rays + 8 * i;
        const int64_t t = tri[i];
        double v0[3], e1[3], e2[3], d[3], org[3];
        for (int k = 0; k < 3; ++k) {
            v0[k] = verts[3 * (int64_t)idx[3 * t] + k];
            e1[k] = (double)verts[3 * (int64_t)idx[3 * t + 1] + k] - v0[k];
            e2[k] = (double)verts[3 * (int64_t)idx[3 * t + 2] + k] - v0[k];
            d[k] = q[4 + k];
            org[k] = q[k];
        }
        double p[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
        double det = e1[0] * p[0] + e1[1] * p[1] + e1[2] * p[2];
        double tv[3] = {org[0] - v0[0], org[1] - v0[1], org[2] - v0[2]};
        double qv[3] = {tv[1] * e1[2] - tv[2] * e1[1], tv[2] * e1[0] - tv[0] * e1[2], tv[0] * e1[1] - tv[1] * e1[0]};
        double inv = 1.0 / det;
        o[1] = (tv[0] * p[0] + tv[1] * p[1] + tv[2] * p[2]) * inv;
        o[2] = (d[0] * qv[0] + d[1] * qv[1] + d[2] * qv[2]) * inv;
        o[0] = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) * inv;
    }
}


/* ---- two-level instancing ------------------------------------------------
 * vr::mat4f (vrbase) is not vendored, so the matrix-vector product is
 * restated with one fixed evaluation order, shared with the GPU library:
 *   x' = ((m[0] x + m[1] y) + m[2] z) + m[3]   (rows of a 3 x 4 matrix)
 * and directions drop the translation column (Transform::inverseTransform,
 * include/rt/Transform.h:31-40). */
static inline void xf_point(const float* m, const float* p, float* o) {
    for (int i = 0; i < 3; ++i) {
        float a = m[4 * i] * p[0];
        float b = m[4 * i + 1] * p[1];
        float c = m[4 * i + 2] * p[2];
        o[i] = ((a + b) + c) + m[4 * i + 3];
    }
}

static inline void xf_dir(const float* m, const float* d, float* o) {
    for (int i = 0; i < 3; ++i) {
        float a = m[4 * i] * d[0];
        float b = m[4 * i + 1] * d[1];
        float c = m[4 * i + 2] * d[2];
        o[i] = (a + b) + c;
    }
}

/* Context::instantiateGeometry (src/rtcore/Context.cpp:366-389): the eight
 * corners of the geometry's box (Aabb::computeVertices order,
 * src/rtcore/Aabb.cpp:124-134) transformed by the instance matrix and added
 * to a default box with Aabb::expandBy(vertex) (if / else-if per axis,
 * src/rtcore/Aabb.cpp:37-53), then Aabb::scaleBy(0.01f) (:78-91). */
void orc_instance_box(const float* gbmin, const float* gbmax, const float* xf, float* bmin, float* bmax) {
    const float c[8][3] = {{gbmin[0], gbmin[1], gbmax[2]}, {gbmax[0], gbmin[1], gbmax[2]},
                           {gbmax[0], gbmin[1], gbmin[2]}, {gbmin[0], gbmin[1], gbmin[2]},
                           {gbmin[0], gbmax[1], gbmax[2]}, {gbmax[0], gbmax[1], gbmax[2]},
                           {gbmax[0], gbmax[1], gbmin[2]}, {gbmin[0], gbmax[1], gbmin[2]}};
    for (int d = 0; d < 3; ++d) {
        bmin[d] = FLT_MAX;
        bmax[d] = -FLT_MAX;
    }
    for (int v = 0; v < 8; ++v) {
        float p[3];
        xf_point(xf, c[v], p);
        for (int d = 0; d < 3; ++d) {
            if (p[d] < bmin[d]) bmin[d] = p[d];
            else if (p[d] > bmax[d]) bmax[d] = p[d];
        }
    }
    for (int d = 0; d < 3; ++d) {
        float sc = (bmin[d] == bmax[d]) ? 0.01f : vabs(bmax[d] - bmin[d]) * 0.01f;
        bmin[d] -= sc;
        bmax[d] += sc;
    }
}

/* IAccStructBuilder::buildInstance (src/rtcore/IAccStructBuilder.cpp:16-33):
 * default box expanded by every instance box (Aabb::expandBy(Aabb),
 * src/rtcore/Aabb.cpp:55-76). */
void orc_scene_box(int32_t ninst, const float* inst_boxes, float* box) {
    for (int d = 0; d < 3; ++d) {
        box[d] = FLT_MAX;
        box[3 + d] = -FLT_MAX;
    }
    for (int32_t i = 0; i < ninst; ++i) {
        for (int d = 0; d < 3; ++d) {
            if (inst_boxes[6 * i + d] < box[d]) box[d] = inst_boxes[6 * i + d];
            if (inst_boxes[6 * i + 3 + d] > box[3 + d]) box[3 + d] = inst_boxes[6 * i + 3 + d];
        }
    }
}

/* IAccStruct::traceNearestInstance (src/rtcore/IAccStruct.cpp:26-72): clip
 * the ray against the scene box; then, instance by instance in order, trace
 * the ray taken to the instance's local space (same tnear / tfar, direction
 * not renormalised) with the best distance so far, so a later instance wins
 * only with a strictly closer hit.  t is the same in both spaces (affine map).
 * The ray's own tnear / tfar words stand for the Context's initialisation
 * (tnear = ray epsilon, tfar = MAX, :34-36).  any != 0: occluded[i] = closest
 * t < the ray's tfar word, as for a single geometry. */
void orc_trace_instances(int32_t ninst, const orc_grid_info* const* g, const int32_t* const* offsets,
                         const int32_t* const* ids, const float* const* acc, const float* inv, const float* box,
                         const float* rays, int64_t n, float* hits, int32_t* inst_out, uint8_t* occluded,
                         int nthreads) {
    orc_grid_info sb;
    memset(&sb, 0, sizeof(sb));
    for (int d = 0; d < 3; ++d) {
        sb.bmin[d] = box[d];
        sb.bmax[d] = box[3 + d];
    }
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
#endif
    for (int64_t i = 0; i < n; ++i) {
        oray w;
        load_ray(rays + 8 * i, &w);
        const float tmax = rays[8 * i + 7];
        float best = FLT_MAX;
        int32_t found = -1;
        ohit hit = {-1, 0.f, 0.f};
        if (clip_ray(&sb, &w)) {
            for (int32_t j = 0; j < ninst; ++j) {
                if (g[j]->ncells <= 0) continue;
                oray r;
                xf_point(inv + 12 * j, w.orig, r.orig);
                xf_dir(inv + 12 * j, w.dir, r.dir);
                r.tnear = w.tnear;
                r.tfar = w.tfar;
                ray_update(&r);
                ohit h = {-1, 0.f, 0.f};
                float t = 0.f;
                if (trace_one_from(g[j], offsets[j], ids[j], acc[j], &r, &h, &t, NULL, NULL, best)) {
                    best = t;
                    found = j;
                    hit = h;
                }
            }
        }
        if (occluded) occluded[i] = (uint8_t)(found >= 0 && best < tmax);
        if (hits) {
            float* o = hits + 4 * i;
            const int32_t id = found >= 0 ? hit.id : -1;
            memcpy(&o[0], &id, 4);
            o[1] = found >= 0 ? best : 0.f;
            o[2] = found >= 0 ? hit.u : 0.f;
            o[3] = found >= 0 ? hit.v : 0.f;
        }
        if (inst_out) inst_out[i] = found;
    }
}

/* ---- shading: the reference's per-pixel recursion ------------------------
 * Context::traceNearest + material / environment shade
 * (src/rtcore/Sample.cpp, src/rtplugins/{HeadlightMaterial,HeadlightMaterialColor,
 * PhongMaterial,PhongMaterialColor,SimplePointLight,SimpleEnvironment}.cpp).
 * Shadow rays are occluded when the closest hit before the light has
 * t < 1 (the GPU shader semantics; the CPU any-hit is a stub).  vr::vec3f is
 * absent from the checkout: normalise = v * (1 / sqrt(v.v)). */
typedef struct { float x, y, z; } ov3;
static inline ov3 o3(float x, float y, float z) { ov3 r = {x, y, z}; return r; }
static inline ov3 oadd(ov3 a, ov3 b) { return o3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline ov3 osub(ov3 a, ov3 b) { return o3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline ov3 osc(ov3 a, float s) { return o3(a.x * s, a.y * s, a.z * s); }
static inline ov3 omul(ov3 a, ov3 b) { return o3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline float odot(ov3 a, ov3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline ov3 onorm(ov3 a) { float inv = 1.0f / sqrtf(odot(a, a)); return osc(a, inv); }
static inline ov3 orefl(ov3 i, ov3 n) { return osub(i, osc(n, odot(i, n) * 2.0f)); }

typedef struct {
    const orc_grid_info* g; const int32_t* offsets; const int32_t* ids; const float* acc;
    const int32_t* idx; const float* normals; const float* colors; const int32_t* material;
    const orc_material* mats; int32_t nmats; const orc_light* lights; int32_t nlights;
    const float* bg; int32_t max_depth; float medium;
} shade_ctx;

static int closest(const shade_ctx* C, ov3 o, ov3 d, float tnear, float tfar, ohit* h, float* t) {
    oray r;
    r.orig[0] = o.x; r.orig[1] = o.y; r.orig[2] = o.z;
    r.dir[0] = d.x; r.dir[1] = d.y; r.dir[2] = d.z;
    r.tnear = tnear;
    r.tfar = tfar;
    ray_update(&r);
    h->id = -1;
    return C->g->ncells > 0 && trace_one(C->g, C->offsets, C->ids, C->acc, &r, h, t, NULL, NULL);
}

static ov3 shade_ray(const shade_ctx* C, ov3 o, ov3 d, int depth, int64_t* nrays) {
    ohit h;
    float t = 0.f;
    ++*nrays;
    if (!closest(C, o, d, 2e-4f, FLT_MAX, &h, &t)) return o3(C->bg[0], C->bg[1], C->bg[2]);
    const int64_t tri = h.id;
    const float b[3] = {1.0f - h.u - h.v, h.u, h.v};
    ov3 n = o3(0.f, 0.f, 0.f), vc = o3(0.f, 0.f, 0.f);
    for (int k = 0; k < 3; ++k) {
        const float* nk = C->normals + 3 * (int64_t)C->idx[3 * tri + k];
        n = oadd(n, osc(o3(nk[0], nk[1], nk[2]), b[k]));
        if (C->colors) {
            const float* ck = C->colors + 3 * (int64_t)C->idx[3 * tri + k];
            vc = oadd(vc, osc(o3(ck[0], ck[1], ck[2]), b[k]));
        }
    }
    if (!C->colors) vc = o3(1.f, 1.f, 1.f);
    n = onorm(n);
    const int m = C->material ? C->material[tri] : 0;
    orc_material M;
    memset(&M, 0, sizeof(M));
    if (m >= 0 && m < C->nmats) M = C->mats[m];
    else { M.type = 0; M.ambient[0] = M.ambient[1] = M.ambient[2] = 0.1f; }
    const ov3 amb = o3(M.ambient[0], M.ambient[1], M.ambient[2]);
    if (M.type == 0 || M.type == 1) {   /* headlight */
        const ov3 c = M.type == 0 ? vc : o3(M.diffuse[0], M.diffuse[1], M.diffuse[2]);
        const float ndd = -odot(n, onorm(d));
        return omul(oadd(amb, osc(osub(c, amb), ndd)), c);
    }
    const ov3 p = oadd(o, osc(d, t));
    const ov3 spec = onorm(orefl(d, n));
    const ov3 hp = oadd(p, osc(n, 2e-4f));
    ov3 dif = o3(0.f, 0.f, 0.f), spc = o3(0.f, 0.f, 0.f);
    for (int i = 0; i < C->nlights; ++i) {
        const orc_light* Lt = &C->lights[i];
        if (odot(n, d) > 0.0f) continue;                      /* back face */
        const ov3 L = osub(o3(Lt->position[0], Lt->position[1], Lt->position[2]), hp);
        if (odot(n, L) <= 0.0f) continue;                     /* initShadowRay */
        if (Lt->cast_shadows) {
            ohit sh;
            float st = 0.f;
            ++*nrays;
            if (closest(C, hp, L, 2e-4f, 1.0f, &sh, &st) && st < 1.0f) continue;
        }
        const ov3 Ld = onorm(L);
        const ov3 lc = o3(Lt->intensity[0], Lt->intensity[1], Lt->intensity[2]);
        dif = oadd(dif, osc(lc, odot(n, Ld)));
        if (M.type == 2 || M.specular_exponent > 0.0f) {
            const float sdl = odot(spec, Ld);
            if (sdl > 0.0f) spc = oadd(spc, osc(lc, powf(sdl, M.specular_exponent)));
        }
    }
    const ov3 sc = o3(M.specular[0], M.specular[1], M.specular[2]);
    ov3 out;
    if (M.type == 2) {
        out = oadd(omul(vc, oadd(amb, dif)), omul(sc, spc));
    } else {
        out = omul(o3(M.diffuse[0], M.diffuse[1], M.diffuse[2]), dif);
        out = oadd(out, oadd(amb, omul(sc, spc)));
    }
    if (depth >= C->max_depth) return out;
    if (M.reflexion > 0.0f) {
        const ov3 rc = shade_ray(C, p, orefl(d, n), depth + 1, nrays);
        out = oadd(out, osc(rc, M.reflexion));
    }
    if (M.opacity < 1.0f) {
        const int front = odot(n, d) <= 0.0f;
        const ov3 nn = front ? n : osc(n, -1.0f);
        const float ratio = front ? C->medium / M.refraction_index : M.refraction_index / C->medium;
        const ov3 nd = onorm(d);
        const float cosI = -odot(nn, nd);
        const float cosT2 = 1.0f - ratio * ratio * (1.0f - cosI * cosI);
        if (cosT2 > 0.0f) {
            const float cosT = sqrtf(cosT2);
            const ov3 td = oadd(osc(nd, ratio), osc(nn, ratio * cosI - cosT));
            const ov3 rc = shade_ray(C, p, td, depth + 1, nrays);
            out = oadd(out, osc(rc, 1.0f - M.opacity));
        }
    }
    return out;
}

int64_t orc_render(const orc_grid_info* g, const int32_t* offsets, const int32_t* ids, const float* acc,
                   const int32_t* idx, const float* normals, const float* colors, const int32_t* material,
                   const orc_material* mats, int32_t nmats, const orc_light* lights, int32_t nlights,
                   const float* background, int32_t max_depth, float medium, const float* primary, int64_t n,
                   float* rgb, int nthreads) {
    shade_ctx C = {g, offsets, ids, acc, idx, normals, colors, material, mats, nmats, lights, nlights,
                   background, max_depth, medium};
    int64_t total = 0;
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt) reduction(+ : total)
#endif
    for (int64_t i = 0; i < n; ++i) {
        const float* q = primary + 8 * i;
        int64_t nr = 0;
        const ov3 c = shade_ray(&C, o3(q[0], q[1], q[2]), o3(q[4], q[5], q[6]), 0, &nr);
        rgb[3 * i] = c.x;
        rgb[3 * i + 1] = c.y;
        rgb[3 * i + 2] = c.z;
        total += nr;
    }
    return total;
}
