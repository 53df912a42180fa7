// gridrt_reference_plugin.hpp -- the reference-side binding of libgridrt.
//
// The reference's own plugin classes, implemented over the C ABI (gridrt.h):
// a maintainer compiles this header inside the reference's tree, against the
// reference's headers (rt/IAccStructBuilder.h, rt/IAccStruct.h, rt/Geometry.h
// and the vr library they include), links libgridrt.so and selects the GPU
// grid with
//     context->setAccStructBuilder(new rtp::GpuUniformGridAccStructBuilder(k));
// (Context::setAccStructBuilder, src/rtcore/Context.cpp:109-112).  From then
// on Context::endGeometry builds every geometry's grid on the GPU
// (src/rtcore/Context.cpp:340-343) and IAccStruct::traceNearestInstance
// (src/rtcore/IAccStruct.cpp:26-72) traces each instance through
// GpuUniformGridAccStruct::traceNearestGeometry.
//
//   rtp::GpuUniformGridAccStructBuilder   replaces rtp::UniformGridAccStructBuilder
//       rt::IAccStructBuilder::buildGeometry        include/rt/IAccStructBuilder.h:16
//       (src/rtplugins/UniformGridAccStructBuilder.cpp:58-149)
//   rtp::GpuUniformGridAccStruct          replaces rtp::UniformGridAccStruct
//       rt::IAccStruct::traceNearestGeometry        include/rt/IAccStruct.h:22
//       rt::IAccStruct::traceAnyGeometry            include/rt/IAccStruct.h:28
//       (src/rtplugins/UniformGridAccStruct.cpp:30-42, 113-196)
//
// Semantics kept from the reference: plugins are intrusively reference
// counted (Geometry::accStruct is a vr::ref_ptr that takes ownership of the
// new structure, and the destructor stays protected as IPlugin's is); the
// calls return void and fail silently -- a failed build leaves a structure
// that reports no hits, lastStatus() gives the rtg_status of the last C-ABI
// call and rtg_last_error() its text; a trace updates the hit only when it is
// closer than hit.distance on entry, and then also sets hit.instance; the
// grid box becomes the structure's bounding box (IAccStruct::_bbox), which
// IAccStruct::traceNearestInstance clips scene rays against.  The any-hit
// call reports occlusion before ray.tfar (the reference's CPU version is a
// stub that returns false, src/rtcore/IAccStruct.cpp:116-122).
//
// A per-ray call costs one GPU round trip: renderers trace whole batches
// with traceNearestBatch / traceAnyBatch (or rtg_trace_frame), as the
// reference's CudaRenderer traces whole frames (src/rtcuda/CudaRenderer.cpp:33-63).
#pragma once

#include <cstdint>
#include <vector>

#include <rt/Geometry.h>
#include <rt/Hit.h>
#include <rt/IAccStruct.h>
#include <rt/IAccStructBuilder.h>
#include <rt/Instance.h>
#include <rt/Ray.h>

#include "gridrt.h"

namespace rtp {

class GpuUniformGridAccStruct : public rt::IAccStruct {
public:
    explicit GpuUniformGridAccStruct(int device = 0) { _status = rtg_scene_create(device, nullptr, &_scene); }

    rtg_scene scene() const { return _scene; }
    rtg_status lastStatus() const { return _status; }
    bool built() const { return _built; }

    virtual void traceNearestGeometry(const rt::Instance& instance, rt::Ray& ray, rt::Hit& hit) {
        if (!_built) return;
        float r[8];
        pack(ray, r);
        rtg_hit h;
        _status = rtg_trace_nearest(_scene, r, 1, &h, 0, nullptr);
        if (_status == RTG_OK) apply(instance, h, hit);
    }

    virtual bool traceAnyGeometry(const rt::Instance&, rt::Ray& ray, rt::Hit&) {
        if (!_built) return false;
        float r[8];
        pack(ray, r);
        uint8_t occ = 0;
        _status = rtg_trace_any(_scene, r, 1, &occ, 0, nullptr);
        return _status == RTG_OK && occ == 1;
    }

    // n rays in one GPU call; hits[i] follows the closer-hit rule per ray.
    void traceNearestBatch(const rt::Instance& instance, const std::vector<rt::Ray>& rays,
                           std::vector<rt::Hit>& hits) {
        hits.resize(rays.size());
        if (!_built || rays.empty()) return;
        std::vector<float> r(8 * rays.size());
        for (size_t i = 0; i < rays.size(); ++i) pack(rays[i], &r[8 * i]);
        std::vector<rtg_hit> h(rays.size());
        _status = rtg_trace_nearest(_scene, r.data(), (int64_t)rays.size(), h.data(), 0, nullptr);
        if (_status != RTG_OK) return;
        for (size_t i = 0; i < rays.size(); ++i) apply(instance, h[i], hits[i]);
    }

    void traceAnyBatch(const std::vector<rt::Ray>& rays, std::vector<uint8_t>& occluded) {
        occluded.assign(rays.size(), 0);
        if (!_built || rays.empty()) return;
        std::vector<float> r(8 * rays.size());
        for (size_t i = 0; i < rays.size(); ++i) pack(rays[i], &r[8 * i]);
        _status = rtg_trace_any(_scene, r.data(), (int64_t)rays.size(), occluded.data(), 0, nullptr);
    }

protected:
    virtual ~GpuUniformGridAccStruct() {
        if (_scene) rtg_scene_destroy(_scene);
    }

private:
    friend class GpuUniformGridAccStructBuilder;

    static void pack(const rt::Ray& ray, float* r) {
        r[0] = ray.orig.x; r[1] = ray.orig.y; r[2] = ray.orig.z; r[3] = ray.tnear;
        r[4] = ray.dir.x; r[5] = ray.dir.y; r[6] = ray.dir.z; r[7] = ray.tfar;
    }

    static void apply(const rt::Instance& instance, const rtg_hit& h, rt::Hit& hit) {
        if (h.id >= 0 && h.t < hit.distance) {
            hit.triangleId = (uint32)h.id;
            hit.distance = h.t;
            hit.v1Coord = h.u;
            hit.v2Coord = h.v;
            hit.v0Coord = 1.0f - h.u - h.v;
            hit.instance = &instance;
        }
    }

    rtg_scene _scene = nullptr;
    rtg_status _status = RTG_OK;
    bool _built = false;
};

// k cells per triangle (the reference hard-codes 6,
// src/rtplugins/UniformGridAccStructBuilder.cpp:91).
class GpuUniformGridAccStructBuilder : public rt::IAccStructBuilder {
public:
    explicit GpuUniformGridAccStructBuilder(int32 k = 6, int device = 0) : _k(k), _device(device) {}

    rtg_status lastStatus() const { return _status; }

    virtual void buildGeometry(rt::Geometry* geometry) {
        GpuUniformGridAccStruct* acc = new GpuUniformGridAccStruct(_device);
        geometry->accStruct = acc;                // the ref_ptr owns it from here
        _status = acc->_status;
        if (_status != RTG_OK) return;
        std::vector<int32_t> tris(3 * geometry->triDesc.size());
        for (size_t t = 0; t < geometry->triDesc.size(); ++t)
            for (int j = 0; j < 3; ++j) tris[3 * t + j] = (int32_t)geometry->triDesc[t].v[j];
        // vr::vec3f holds three packed floats: the vertex array is float[3 V]
        const float* v = geometry->vertices.empty() ? nullptr : &geometry->vertices[0].x;
        _status = rtg_scene_set_geometry(acc->_scene, v, (int64_t)geometry->vertices.size(),
                                         tris.empty() ? nullptr : tris.data(), (int64_t)geometry->triDesc.size(),
                                         nullptr);
        if (_status == RTG_OK) _status = rtg_scene_build(acc->_scene, _k, nullptr);
        acc->_status = _status;
        if (_status != RTG_OK) return;
        rtg_grid_info gi;
        _status = rtg_scene_grid_info(acc->_scene, &gi);
        if (_status != RTG_OK) return;
        rt::Aabb box;
        box.minv.set(gi.bmin[0], gi.bmin[1], gi.bmin[2]);
        box.maxv.set(gi.bmax[0], gi.bmax[1], gi.bmax[2]);
        acc->setBoundingBox(box);
        acc->_built = true;
    }

private:
    int32 _k;
    int _device;
    rtg_status _status = RTG_OK;
};

}  // namespace rtp
