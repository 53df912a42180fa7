/*
 * oracle/ref_api.cpp -- C entry points over the reference's OWN CPU code.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
 * the unmodified reference sources (read in place from the reference checkout)
 * and the `vr` shim into oracle/_ref/liboracle_ref.so.  Only tests and the
 * golden-fixture generator load it; the product never does.
 *
 * What it drives (paths relative to the reference project):
 *   rtp::UniformGridAccStructBuilder::buildGeometry
 *       src/rtplugins/UniformGridAccStructBuilder.cpp:58-149  (k = 6 fixed)
 *   rtp::UniformGridAccStruct::traceNearestGeometry / traverse3ddda
 *       src/rtplugins/UniformGridAccStruct.cpp:30-42, 113-196
 *   rt::IAccStruct::traceNearestGeometry (brute force over all triangles)
 *       src/rtcore/IAccStruct.cpp:74-106
 *   rt::TriAccel::buildFrom / valid   src/rtcore/Triangle.cpp:11-63
 * Geometry is filled the way PrimitiveBuilder::storeValidTriangle does
 * (src/rtcore/PrimitiveBuilder.cpp:120-128): invalid triangles are rejected
 * (this harness returns an error instead of renumbering).
 */
#include <rt/Geometry.h>
#include <rt/Instance.h>
#include <rt/Ray.h>
#include <rt/Hit.h>
#include <rtp/UniformGridAccStruct.h>
#include <rtp/UniformGridAccStructBuilder.h>

#include <cstdint>
#include <fcntl.h>
#include <unistd.h>
#include <cstdio>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {
struct RefScene {
    vr::ref_ptr<rt::Geometry> geom;
    rt::Instance inst;
    rtp::UniformGridAccStruct* grid = nullptr;
};
}  // namespace

extern "C" {

/* Returns NULL when a triangle is invalid (TriAccel::valid() false) or an
 * index is out of range.  `quiet` redirects the builder's stats printf. */
void* ref_scene_create(const float* verts, int64_t nverts, const int32_t* idx, int64_t ntris, int quiet) {
    RefScene* s = new RefScene();
    s->geom = new rt::Geometry();
    rt::Geometry& g = *s->geom;
    g.vertices.resize((size_t)nverts);
    for (int64_t i = 0; i < nverts; ++i) g.vertices[i].set(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
    for (int64_t t = 0; t < ntris; ++t) {
        rt::TriDesc d;
        for (int k = 0; k < 3; ++k) {
            int32_t v = idx[3 * t + k];
            if (v < 0 || v >= nverts) { delete s; return nullptr; }
            d.v[k] = (uint32)v;
        }
        rt::TriAccel acc;
        acc.buildFrom(g.vertices[d.v[0]], g.vertices[d.v[1]], g.vertices[d.v[2]]);
        if (!acc.valid()) { delete s; return nullptr; }
        acc.triangleId = (uint32)g.triDesc.size();
        g.triDesc.push_back(d);
        g.triAccel.push_back(acc);
    }
    fflush(stdout);
    int saved_fd = -1;
    if (quiet) {
        saved_fd = dup(1);
        int nul = open("/dev/null", O_WRONLY);
        if (nul >= 0) { dup2(nul, 1); close(nul); }
    }
    rtp::UniformGridAccStructBuilder builder;
    builder.buildGeometry(s->geom.get());
    fflush(stdout);
    if (saved_fd >= 0) { dup2(saved_fd, 1); close(saved_fd); }
    s->grid = dynamic_cast<rtp::UniformGridAccStruct*>(g.accStruct.get());
    s->inst.geometry = s->geom.get();
    return s;
}

void ref_scene_destroy(void* h) { delete static_cast<RefScene*>(h); }

/* res[3], bbox[6] (min xyz, max xyz), cell[3], inv_cell[3], *nrefs */
void ref_scene_grid_info(void* h, int32_t* res, float* bbox, float* cell, float* inv_cell, int64_t* nrefs) {
    RefScene* s = static_cast<RefScene*>(h);
    int32 nx, ny, nz;
    s->grid->getResolution(nx, ny, nz);
    res[0] = nx; res[1] = ny; res[2] = nz;
    const rt::Aabb& b = s->grid->getBoundingBox();
    for (int k = 0; k < 3; ++k) {
        bbox[k] = b.minv[k];
        bbox[3 + k] = b.maxv[k];
        cell[k] = s->grid->getCellSize()[k];
        inv_cell[k] = s->grid->getInvCellSize()[k];
    }
    int64_t r = 0;
    for (const auto& c : s->grid->getGridData()) r += (int64_t)c.size();
    *nrefs = r;
}

/* CSR flattening in linear cell order x + y*nx + z*nx*ny (the same order as
 * src/rtcuda/CudaRenderer.cpp:172-196, without the *3 vertex scaling). */
void ref_scene_grid_csr(void* h, int32_t* offsets, int32_t* ids) {
    RefScene* s = static_cast<RefScene*>(h);
    const auto& data = s->grid->getGridData();
    int64_t pos = 0;
    for (size_t c = 0; c < data.size(); ++c) {
        offsets[c] = (int32_t)pos;
        for (int32 t : data[c]) ids[pos++] = t;
    }
    offsets[data.size()] = (int32_t)pos;
}

/* rays: n x 8 floats {ox, oy, oz, tnear, dx, dy, dz, tfar}
 * hits: n x 4 {id (int32 bits, -1 = miss), t, u (v1Coord), v (v2Coord)}
 * brute != 0 uses the base-class brute-force traversal instead of the grid. */
void ref_scene_trace(void* h, const float* rays, int64_t n, float* hits, int brute, int nthreads) {
    RefScene* s = static_cast<RefScene*>(h);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (int64_t i = 0; i < n; ++i) {
        const float* r = rays + 8 * i;
        rt::Ray ray;
        ray.orig.set(r[0], r[1], r[2]);
        ray.dir.set(r[4], r[5], r[6]);
        ray.tnear = r[3];
        ray.tfar = r[7];
        ray.update();
        rt::Hit hit;
        hit.instance = nullptr;
        hit.distance = vr::Mathf::MAX_VALUE;
        hit.triangleId = 0xFFFFFFFFu;
        hit.v0Coord = hit.v1Coord = hit.v2Coord = 0.f;
        if (brute)
            s->grid->rt::IAccStruct::traceNearestGeometry(s->inst, ray, hit);
        else
            s->grid->traceNearestGeometry(s->inst, ray, hit);
        int32_t id = hit.instance ? (int32_t)hit.triangleId : -1;
        float* o = hits + 4 * i;
        std::memcpy(&o[0], &id, 4);
        o[1] = hit.instance ? hit.distance : 0.f;
        o[2] = hit.instance ? hit.v1Coord : 0.f;
        o[3] = hit.instance ? hit.v2Coord : 0.f;
    }
}

/* TriAccel records as built by the reference: n x 12 words (k, n_u, n_v, n_d,
 * b_nu, b_nv, b_d, pad, c_nu, c_nv, c_d, triangleId). */
void ref_scene_triaccel(void* h, float* out) {
    RefScene* s = static_cast<RefScene*>(h);
    const auto& ta = s->geom->triAccel;
    for (size_t t = 0; t < ta.size(); ++t) std::memcpy(out + 12 * t, &ta[t], 48);
}

}  // extern "C"
