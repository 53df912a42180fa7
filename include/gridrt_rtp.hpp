// gridrt_rtp.hpp -- C++ mirror of the reference's acceleration-structure
// plugin interface, implemented over the C ABI (gridrt.h).
//
// Mirrors, with the same names and argument meaning:
//   rt::Ray, rt::Hit, rt::TriDesc, rt::Geometry, rt::Instance
//       include/rt/Ray.h:9-24, include/rt/Hit.h:9-17, include/rt/Triangle.h:15-20,
//       include/rt/Geometry.h:10-27, include/rt/Instance.h:11-18
//   rt::IAccStructBuilder::buildGeometry(Geometry*)       include/rt/IAccStructBuilder.h:12-18
//   rt::IAccStruct::traceNearestGeometry / traceAnyGeometry include/rt/IAccStruct.h:10-32
//   rtp::UniformGridAccStructBuilder / UniformGridAccStruct (the grid plugin pair)
//       include/rtp/UniformGridAccStructBuilder.h, include/rtp/UniformGridAccStruct.h
//   the scene level, rtp::InstancedScene: IAccStructBuilder::buildInstance +
//       IAccStruct::traceNearestInstance (include/rt/IAccStructBuilder.h:17, include/rt/IAccStruct.h:19)
// Error behaviour follows the reference: the calls return void and fail
// silently (a failed build leaves an acceleration structure that reports no
// hits); lastStatus() exposes the rtg_status of the last C-ABI call.
//
// Per-ray calls are correct but pay one GPU round trip each; renderers use
// the batched traceNearestBatch / traceAnyBatch or GpuFrameRenderer, as the
// reference's CudaRenderer traces whole frames (src/rtcuda/CudaRenderer.cpp:33-63).
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "gridrt.h"

namespace gridrt {
namespace rt {

struct vec3f {
    float x = 0.f, y = 0.f, z = 0.f;
    vec3f() = default;
    vec3f(float a, float b, float c) : x(a), y(b), z(c) {}
    float& operator[](int i) { return (&x)[i]; }
    float operator[](int i) const { return (&x)[i]; }
};

struct Ray {
    vec3f orig;
    vec3f dir;
    float tnear = 2e-4f;                  // Context::getRayEpsilon default, src/rtcore/Context.cpp:505
    float tfar = 3.402823466e+38f;        // vr::Mathf::MAX_VALUE
};

struct Instance;

struct Hit {
    uint32_t triangleId = 0xffffffffu;
    float v0Coord = 0.f, v1Coord = 0.f, v2Coord = 0.f;
    float distance = 3.402823466e+38f;
    const Instance* instance = nullptr;   // set on a hit, as the reference does
};

struct TriDesc {
    uint32_t v[3];
};

class IAccStruct;

struct Geometry {
    std::vector<vec3f> vertices;
    std::vector<TriDesc> triDesc;
    std::shared_ptr<IAccStruct> accStruct;
};

// rt::Instance with rt::Transform's two matrices (include/rt/Instance.h:13-18,
// include/rt/Transform.h:10-29) as 3 x 4 row-major arrays.
struct Instance {
    Geometry* geometry = nullptr;
    float worldFromLocal[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    float localFromWorld[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
};

class IAccStruct {
public:
    virtual ~IAccStruct() = default;
    virtual void traceNearestGeometry(const Instance& instance, Ray& ray, Hit& hit) = 0;
    virtual bool traceAnyGeometry(const Instance& instance, Ray& ray, Hit& hit) = 0;
};

class IAccStructBuilder {
public:
    virtual ~IAccStructBuilder() = default;
    virtual void buildGeometry(Geometry* geometry) = 0;
};

}  // namespace rt

namespace rtp {

// The GPU grid behind one Geometry (the role of rtp::UniformGridAccStruct).
class UniformGridAccStruct : public rt::IAccStruct {
public:
    explicit UniformGridAccStruct(int device = 0) { _status = rtg_scene_create(device, nullptr, &_scene); }
    ~UniformGridAccStruct() override { rtg_scene_destroy(_scene); }
    UniformGridAccStruct(const UniformGridAccStruct&) = delete;
    UniformGridAccStruct& operator=(const UniformGridAccStruct&) = delete;

    rtg_scene scene() const { return _scene; }
    rtg_status lastStatus() const { return _status; }

    // rt::IAccStruct::traceNearestGeometry: updates hit only when a closer
    // hit than hit.distance is found (src/rtplugins/UniformGridAccStruct.cpp:157,169-174).
    void traceNearestGeometry(const rt::Instance& instance, rt::Ray& ray, rt::Hit& hit) override {
        float r[8] = {ray.orig.x, ray.orig.y, ray.orig.z, ray.tnear, ray.dir.x, ray.dir.y, ray.dir.z, ray.tfar};
        rtg_hit h;
        _status = rtg_trace_nearest(_scene, r, 1, &h, 0, nullptr);
        if (_status == RTG_OK) apply(instance, h, hit);
    }

    // Occlusion before ray.tfar (the reference's CPU version is a stub that
    // returns false, src/rtcore/IAccStruct.cpp:116-122).
    bool traceAnyGeometry(const rt::Instance&, rt::Ray& ray, rt::Hit&) override {
        float r[8] = {ray.orig.x, ray.orig.y, ray.orig.z, ray.tnear, ray.dir.x, ray.dir.y, ray.dir.z, ray.tfar};
        uint8_t occ = 0;
        _status = rtg_trace_any(_scene, r, 1, &occ, 0, nullptr);
        return _status == RTG_OK && occ == 1;
    }

    // Batched forms: one GPU call for all rays.
    void traceNearestBatch(const rt::Instance& instance, std::vector<rt::Ray>& rays, std::vector<rt::Hit>& hits) {
        std::vector<float> r = pack(rays);
        std::vector<rtg_hit> h(rays.size());
        hits.resize(rays.size());
        _status = rtg_trace_nearest(_scene, r.data(), (int64_t)rays.size(), h.data(), 0, nullptr);
        if (_status != RTG_OK) return;
        for (size_t i = 0; i < rays.size(); ++i) apply(instance, h[i], hits[i]);
    }

    void traceAnyBatch(std::vector<rt::Ray>& rays, std::vector<uint8_t>& occluded) {
        std::vector<float> r = pack(rays);
        occluded.assign(rays.size(), 0);
        _status = rtg_trace_any(_scene, r.data(), (int64_t)rays.size(), occluded.data(), 0, nullptr);
    }

    // Grid description (UniformGridAccStruct::getResolution / getCellSize ...).
    rtg_grid_info gridInfo() const {
        rtg_grid_info gi;
        rtg_scene_grid_info(_scene, &gi);
        return gi;
    }

private:
    friend class UniformGridAccStructBuilder;

    static std::vector<float> pack(const std::vector<rt::Ray>& rays) {
        std::vector<float> r(rays.size() * 8);
        for (size_t i = 0; i < rays.size(); ++i) {
            const rt::Ray& q = rays[i];
            float* o = &r[8 * i];
            o[0] = q.orig.x; o[1] = q.orig.y; o[2] = q.orig.z; o[3] = q.tnear;
            o[4] = q.dir.x; o[5] = q.dir.y; o[6] = q.dir.z; o[7] = q.tfar;
        }
        return r;
    }

    static void apply(const rt::Instance& instance, const rtg_hit& h, rt::Hit& hit) {
        if (h.id >= 0 && h.t < hit.distance) {
            hit.triangleId = (uint32_t)h.id;
            hit.distance = h.t;
            hit.v1Coord = h.u;
            hit.v2Coord = h.v;
            hit.v0Coord = 1.0f - h.u - h.v;
            hit.instance = &instance;
        }
    }

    rtg_scene _scene = nullptr;
    rtg_status _status = RTG_OK;
};

// The role of rtp::UniformGridAccStructBuilder: builds the grid of a Geometry
// on the GPU with k cells per triangle (the reference hard-codes 6,
// src/rtplugins/UniformGridAccStructBuilder.cpp:91).
class UniformGridAccStructBuilder : public rt::IAccStructBuilder {
public:
    explicit UniformGridAccStructBuilder(int32_t k = 6, int device = 0) : _k(k), _device(device) {}

    void buildGeometry(rt::Geometry* geometry) override {
        auto acc = std::make_shared<UniformGridAccStruct>(_device);
        geometry->accStruct = acc;
        std::vector<int32_t> tris(3 * geometry->triDesc.size());
        for (size_t t = 0; t < geometry->triDesc.size(); ++t)
            for (int j = 0; j < 3; ++j) tris[3 * t + j] = (int32_t)geometry->triDesc[t].v[j];
        _status = acc->_status;
        if (_status != RTG_OK) return;
        const float* v = geometry->vertices.empty() ? nullptr : &geometry->vertices[0].x;
        _status = rtg_scene_set_geometry(acc->scene(), v, (int64_t)geometry->vertices.size(), tris.data(),
                                         (int64_t)geometry->triDesc.size(), nullptr);
        if (_status == RTG_OK) _status = rtg_scene_build(acc->scene(), _k, nullptr);
        acc->_status = _status;
    }

    rtg_status lastStatus() const { return _status; }

private:
    int32_t _k;
    int _device;
    rtg_status _status = RTG_OK;
};

// The scene level: IAccStructBuilder::buildInstance + IAccStruct::traceNearestInstance
// (src/rtcore/IAccStructBuilder.cpp:16-33, src/rtcore/IAccStruct.cpp:26-72) over
// instances whose geometries were built by UniformGridAccStructBuilder.
class InstancedScene {
public:
    InstancedScene() = default;
    ~InstancedScene() { rtg_instances_destroy(_set); }
    InstancedScene(const InstancedScene&) = delete;
    InstancedScene& operator=(const InstancedScene&) = delete;

    rtg_status lastStatus() const { return _status; }

    void buildInstance(const std::vector<rt::Instance>& instances) {
        _instances = instances;
        std::vector<rtg_instance> v(instances.size());
        for (size_t i = 0; i < instances.size(); ++i) {
            auto* acc = dynamic_cast<UniformGridAccStruct*>(instances[i].geometry->accStruct.get());
            if (!acc) {
                _status = RTG_NOT_BUILT;
                return;
            }
            v[i].scene = acc->scene();
            for (int k = 0; k < 12; ++k) {
                v[i].world_from_local[k] = instances[i].worldFromLocal[k];
                v[i].local_from_world[k] = instances[i].localFromWorld[k];
            }
        }
        rtg_instances_destroy(_set);
        _set = nullptr;
        _status = rtg_instances_create(v.data(), (int32_t)v.size(), &_set);
    }

    // traceNearestInstance for a batch of rays: hits[i].instance points into
    // the vector given to buildInstance.
    void traceNearestInstance(std::vector<rt::Ray>& rays, std::vector<rt::Hit>& hits) {
        std::vector<float> r(rays.size() * 8);
        for (size_t i = 0; i < rays.size(); ++i) {
            const rt::Ray& q = rays[i];
            float* o = &r[8 * i];
            o[0] = q.orig.x; o[1] = q.orig.y; o[2] = q.orig.z; o[3] = q.tnear;
            o[4] = q.dir.x; o[5] = q.dir.y; o[6] = q.dir.z; o[7] = q.tfar;
        }
        std::vector<rtg_hit> h(rays.size());
        std::vector<int32_t> inst(rays.size());
        hits.assign(rays.size(), rt::Hit());
        _status = rtg_trace_nearest_instances(_set, r.data(), (int64_t)rays.size(), h.data(), inst.data(), nullptr);
        if (_status != RTG_OK) return;
        for (size_t i = 0; i < rays.size(); ++i) {
            if (h[i].id < 0) continue;
            rt::Hit& o = hits[i];
            o.triangleId = (uint32_t)h[i].id;
            o.distance = h[i].t;
            o.v1Coord = h[i].u;
            o.v2Coord = h[i].v;
            o.v0Coord = 1.0f - h[i].u - h[i].v;
            o.instance = &_instances[inst[i]];
        }
    }

private:
    std::vector<rt::Instance> _instances;
    rtg_instances _set = nullptr;
    rtg_status _status = RTG_OK;
};

// Headless frame tracer in the role of rtc::CudaRenderer (include/rtc/CudaRenderer.h:10-22):
// camera parameters as cudaSetCameraParameters takes them, one call per frame.
class GpuFrameRenderer {
public:
    // hits[w*h] and occluded[w*h] (0 lit, 1 shadowed, 2 no shadow ray).
    static rtg_status render(UniformGridAccStruct& acc, const rtg_camera& cam, const float light[3],
                             std::vector<rtg_hit>& hits, std::vector<uint8_t>& occluded) {
        const size_t n = (size_t)cam.width * (size_t)cam.height;
        hits.resize(n);
        occluded.resize(n);
        return rtg_trace_frame(acc.scene(), &cam, light, hits.data(), occluded.data(), nullptr);
    }
};

// The same frames in a render loop, the read-back of frame f overlapped with
// frame f + 1 (rtg_trace_frame_async): begin() enqueues a frame into one of
// two host buffer pairs and returns its ticket; finish() waits for that
// frame and exposes its buffers, valid until the frame two later begins, so
// finish frame f before beginning frame f + 2.  The copies overlap the next
// frame when the host memory is pinned; with this std::vector storage they
// are correct but the driver copies them synchronously.
class GpuFrameStream {
public:
    explicit GpuFrameStream(UniformGridAccStruct& acc) : _acc(acc) {}

    rtg_status begin(const rtg_camera& cam, const float light[3], uint64_t* ticket) {
        const size_t n = (size_t)cam.width * (size_t)cam.height;
        const int slot = (int)(_begun & 1);
        _hits[slot].resize(n);
        _occ[slot].resize(n);
        const rtg_status rc = rtg_trace_frame_async(_acc.scene(), &cam, light, _hits[slot].data(),
                                                    _occ[slot].data(), nullptr, ticket);
        if (rc == RTG_OK) {
            _ticket[slot] = *ticket;
            ++_begun;
        }
        return rc;
    }

    rtg_status finish(uint64_t ticket, const std::vector<rtg_hit>** hits, const std::vector<uint8_t>** occluded) {
        const int slot = (_begun > 0 && _ticket[(_begun - 1) & 1] == ticket) ? (int)((_begun - 1) & 1)
                                                                             : (int)(_begun & 1);
        if (_begun == 0 || _ticket[slot] != ticket) return RTG_INVALID_PARAM;
        const rtg_status rc = rtg_trace_frame_wait(_acc.scene(), ticket);
        if (rc == RTG_OK) {
            *hits = &_hits[slot];
            *occluded = &_occ[slot];
        }
        return rc;
    }

private:
    UniformGridAccStruct& _acc;
    std::vector<rtg_hit> _hits[2];
    std::vector<uint8_t> _occ[2];
    uint64_t _ticket[2] = {~0ull, ~0ull};
    uint64_t _begun = 0;
};

}  // namespace rtp
}  // namespace gridrt
