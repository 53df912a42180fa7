// instances.cu -- two-level instancing over built scenes (C ABI).
//
// Replaces the scene level of the reference's plugin interface:
//   Context::instantiateGeometry   instance world box (src/rtcore/Context.cpp:352-390)
//   IAccStructBuilder::buildInstance  scene box over all instances (src/rtcore/IAccStructBuilder.cpp:16-33)
//   IAccStruct::traceNearestInstance  per-instance trace in local space (src/rtcore/IAccStruct.cpp:26-72)
// The trace itself is one persistent launch (trace.cu: trace_instances_kernel).
//
// Matrices are 3 x 4, row-major; rows are applied as
// x' = ((m0 x + m1 y) + m2 z) + m3 with one rounding per operation (the
// reference's vr::mat4f is not part of its checkout, so this order is the
// library's definition, shared with the device kernel).
#include <cstring>
#include <string>
#include <vector>

#include "scene.h"

using namespace gridrt;

struct rtg_instances_s {
    int device = 0;
    int num_sms = 0;
    std::vector<rtg_scene> scenes;
    std::vector<float> xf;            // world_from_local, 12 per instance
    std::vector<float> boxes;         // world boxes, 6 per instance
    std::vector<InstanceRec> h_recs;
    InstanceRec* d_recs = nullptr;
    void* d_params = nullptr;         // per-instance grid parameters (filled per launch)
    unsigned long long* d_counter = nullptr;   // ring of per-launch ray counters
    unsigned seq = 0;
    InstanceBox box{};
    TraceTuning tune;
};

namespace {

constexpr unsigned kInstCounters = 32;

rtg_status ifail(rtg_status s, const char* msg) {
    set_last_error(msg);
    return s;
}

#define ITRY(expr)                                                                                 \
    do {                                                                                           \
        cudaError_t _e = (expr);                                                                   \
        if (_e != cudaSuccess) {                                                                   \
            set_last_error(std::string(#expr) + ": " + cudaGetErrorString(_e));                    \
            return _e == cudaErrorMemoryAllocation ? RTG_NO_MEMORY : RTG_DEVICE_ERROR;             \
        }                                                                                          \
    } while (0)

void xf_point_host(const float* m, const float* p, float* o) {
    for (int i = 0; i < 3; ++i) {
        const float a = m[4 * i] * p[0];
        const float b = m[4 * i + 1] * p[1];
        const float c = m[4 * i + 2] * p[2];
        o[i] = ((a + b) + c) + m[4 * i + 3];
    }
}

// Context::instantiateGeometry: the geometry box's corners in
// Aabb::computeVertices order (src/rtcore/Aabb.cpp:124-134), transformed and
// added to a default box by Aabb::expandBy(vertex) -- if / else-if per axis,
// as the reference does (src/rtcore/Aabb.cpp:37-53) -- then scaleBy(0.01f)
// (:78-91).  A degenerate geometry box is kept as it is (Context.cpp:370-374).
void instance_box(const float* gmin, const float* gmax, const float* m, float* out) {
    float* bmin = out;
    float* bmax = out + 3;
    for (int d = 0; d < 3; ++d) {
        bmin[d] = kFltMax;
        bmax[d] = -kFltMax;
    }
    if (gmin[0] > gmax[0] || gmin[1] > gmax[1] || gmin[2] > gmax[2]) return;
    const float c[8][3] = {{gmin[0], gmin[1], gmax[2]}, {gmax[0], gmin[1], gmax[2]}, {gmax[0], gmin[1], gmin[2]},
                           {gmin[0], gmin[1], gmin[2]}, {gmin[0], gmax[1], gmax[2]}, {gmax[0], gmax[1], gmax[2]},
                           {gmax[0], gmax[1], gmin[2]}, {gmin[0], gmax[1], gmin[2]}};
    for (int v = 0; v < 8; ++v) {
        float p[3];
        xf_point_host(m, c[v], p);
        for (int d = 0; d < 3; ++d) {
            if (p[d] < bmin[d]) bmin[d] = p[d];
            else if (p[d] > bmax[d]) bmax[d] = p[d];
        }
    }
    for (int d = 0; d < 3; ++d) {
        const float s = (bmin[d] == bmax[d]) ? 0.01f : std::fabs(bmax[d] - bmin[d]) * 0.01f;
        bmin[d] -= s;
        bmax[d] += s;
    }
}

// Grid box of a built scene, read from the device (a build may have been
// enqueued asynchronously).
rtg_status scene_box(rtg_scene s, float* gmin, float* gmax, bool* empty) {
    GridParams p;
    ITRY(cudaStreamSynchronize(s->stream));
    ITRY(cudaMemcpy(&p, s->d_params, sizeof(GridParams), cudaMemcpyDeviceToHost));
    *empty = s->ntris == 0 || p.ncells <= 0 || build_failed(p.status);
    for (int d = 0; d < 3; ++d) {
        gmin[d] = *empty ? kFltMax : p.bmin[d];
        gmax[d] = *empty ? -kFltMax : p.bmax[d];
    }
    return RTG_OK;
}

rtg_status load(rtg_instances set, const rtg_instance* inst, int32_t n) {
    set->scenes.resize(n);
    set->xf.resize(12 * (size_t)n);
    set->boxes.resize(6 * (size_t)n);
    set->h_recs.resize(n);
    for (int d = 0; d < 3; ++d) {
        set->box.bmin[d] = kFltMax;
        set->box.bmax[d] = -kFltMax;
    }
    for (int32_t i = 0; i < n; ++i) {
        rtg_scene s = inst[i].scene;
        set->scenes[i] = s;
        std::memcpy(&set->xf[12 * (size_t)i], inst[i].world_from_local, 12 * sizeof(float));
        float gmin[3], gmax[3];
        bool empty = false;
        rtg_status rc = scene_box(s, gmin, gmax, &empty);
        if (rc) return rc;
        float* b = &set->boxes[6 * (size_t)i];
        instance_box(gmin, gmax, inst[i].world_from_local, b);
        // IAccStructBuilder::buildInstance: Aabb::expandBy(Aabb) per instance
        for (int d = 0; d < 3; ++d) {
            if (b[d] < set->box.bmin[d]) set->box.bmin[d] = b[d];
            if (b[3 + d] > set->box.bmax[d]) set->box.bmax[d] = b[3 + d];
        }
        InstanceRec& R = set->h_recs[i];
        std::memset(&R, 0, sizeof(R));
        R.view = scene_view(s);
        std::memcpy(R.xf, inst[i].local_from_world, 12 * sizeof(float));
        R.skip = empty ? 1 : 0;
    }
    return RTG_OK;
}

rtg_status upload(rtg_instances set, cudaStream_t st) {
    ITRY(cudaMemcpyAsync(set->d_recs, set->h_recs.data(), sizeof(InstanceRec) * set->h_recs.size(),
                         cudaMemcpyHostToDevice, st));
    ITRY(cudaStreamSynchronize(st));   // the host table may change before the copy ran otherwise
    return RTG_OK;
}

// Scene buffers move when a later build grows them: refresh the table first.
rtg_status refresh_views(rtg_instances set, cudaStream_t st) {
    bool changed = false;
    for (size_t i = 0; i < set->scenes.size(); ++i) {
        const SceneView v = scene_view(set->scenes[i]);
        if (std::memcmp(&v, &set->h_recs[i].view, sizeof(SceneView)) != 0) {
            set->h_recs[i].view = v;
            changed = true;
        }
    }
    return changed ? upload(set, st) : RTG_OK;
}

rtg_status check_args(const rtg_instance* inst, int32_t n, int* device) {
    if (!inst || n <= 0) return ifail(RTG_INVALID_PARAM, "instances: need at least one instance");
    for (int32_t i = 0; i < n; ++i) {
        rtg_scene s = inst[i].scene;
        if (!s) return ifail(RTG_INVALID_PARAM, "instances: NULL scene");
        if (!s->built) return ifail(RTG_NOT_BUILT, "instances: scene not built");
        if (i == 0) *device = s->device;
        else if (s->device != *device) return ifail(RTG_INVALID_PARAM, "instances: scenes on different devices");
    }
    return RTG_OK;
}

}  // namespace

extern "C" {

rtg_status rtg_instances_create(const rtg_instance* inst, int32_t n, rtg_instances* out) {
    if (!out) return ifail(RTG_INVALID_PARAM, "out is NULL");
    *out = nullptr;
    int dev = 0;
    rtg_status rc = check_args(inst, n, &dev);
    if (rc) return rc;
    ITRY(cudaSetDevice(dev));
    rtg_instances set = new rtg_instances_s;
    set->device = dev;
    set->num_sms = inst[0].scene->num_sms;
    set->tune = inst[0].scene->tune;
    if (cudaMalloc(&set->d_recs, sizeof(InstanceRec) * (size_t)n) != cudaSuccess ||
        cudaMalloc(&set->d_params, instance_params_bytes(n)) != cudaSuccess ||
        cudaMalloc(&set->d_counter, sizeof(unsigned long long) * kInstCounters) != cudaSuccess) {
        rtg_instances_destroy(set);
        return ifail(RTG_NO_MEMORY, "instances: device tables");
    }
    rc = load(set, inst, n);
    if (rc == RTG_OK) rc = upload(set, inst[0].scene->stream);
    if (rc) {
        rtg_instances_destroy(set);
        return rc;
    }
    *out = set;
    return RTG_OK;
}

rtg_status rtg_instances_update(rtg_instances set, const rtg_instance* inst, int32_t n) {
    if (!set) return ifail(RTG_INVALID_PARAM, "instance set is NULL");
    if (n != (int32_t)set->scenes.size()) return ifail(RTG_INVALID_PARAM, "instances: count differs from create");
    int dev = 0;
    rtg_status rc = check_args(inst, n, &dev);
    if (rc) return rc;
    if (dev != set->device) return ifail(RTG_INVALID_PARAM, "instances: scenes on a different device");
    ITRY(cudaSetDevice(dev));
    ITRY(cudaDeviceSynchronize());   // traces in flight read the table
    rc = load(set, inst, n);
    if (rc) return rc;
    return upload(set, inst[0].scene->stream);
}

rtg_status rtg_instances_box(rtg_instances set, float box[6], float* inst_boxes) {
    if (!set || !box) return ifail(RTG_INVALID_PARAM, "NULL argument");
    for (int d = 0; d < 3; ++d) {
        box[d] = set->box.bmin[d];
        box[3 + d] = set->box.bmax[d];
    }
    if (inst_boxes) std::memcpy(inst_boxes, set->boxes.data(), sizeof(float) * set->boxes.size());
    return RTG_OK;
}

rtg_status rtg_instances_set_tuning(rtg_instances set, int32_t key, int32_t value) {
    if (!set) return ifail(RTG_INVALID_PARAM, "instance set is NULL");
    if (key == RTG_TUNE_EMPTY_RUN) {
        if (value != 2 && value != 4 && value != 8) return ifail(RTG_INVALID_PARAM, "empty run must be 2, 4 or 8");
        set->tune.empty_run = value;
        return RTG_OK;
    }
    if (key == RTG_TUNE_PERSISTENT) {
        set->tune.persistent = value ? 1 : 0;
        return RTG_OK;
    }
    return ifail(RTG_INVALID_PARAM, "unknown tuning key for an instance set");
}

static rtg_status trace_instances(rtg_instances set, const float* d_rays, int64_t n, rtg_hit* d_hits,
                                  int32_t* d_instance, uint8_t* d_occ, int mode, int32_t flags, void* stream) {
    if (!set) return ifail(RTG_INVALID_PARAM, "instance set is NULL");
    if (n < 0) return ifail(RTG_INVALID_PARAM, "negative ray count");
    if (flags != 0) return ifail(RTG_INVALID_PARAM, "instance traces take no flags");
    if (n == 0) return RTG_OK;
    if (!d_rays || (mode == 0 && !d_hits) || (mode == 1 && !d_occ)) return ifail(RTG_INVALID_PARAM, "NULL arrays");
    ITRY(cudaSetDevice(set->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : set->scenes[0]->stream;
    rtg_status rc = refresh_views(set, st);
    if (rc) return rc;
    const unsigned slot = __atomic_fetch_add(&set->seq, 1u, __ATOMIC_RELAXED) % kInstCounters;
    launch_trace_instances(set->d_recs, set->d_params, (int)set->scenes.size(), set->box,
                           reinterpret_cast<const float4*>(d_rays), n, reinterpret_cast<int4*>(d_hits), d_instance,
                           d_occ, mode, nullptr, set->d_counter + slot, set->tune, set->num_sms, st);
    ITRY(cudaGetLastError());
    return RTG_OK;
}

rtg_status rtg_trace_nearest_instances_device(rtg_instances set, const float* d_rays, int64_t n, rtg_hit* d_hits,
                                              int32_t* d_instance, int32_t flags, void* stream) {
    return trace_instances(set, d_rays, n, d_hits, d_instance, nullptr, 0, flags, stream);
}

rtg_status rtg_trace_any_instances_device(rtg_instances set, const float* d_rays, int64_t n, uint8_t* d_occ,
                                          int32_t flags, void* stream) {
    return trace_instances(set, d_rays, n, nullptr, nullptr, d_occ, 1, flags, stream);
}

rtg_status rtg_trace_nearest_instances(rtg_instances set, const float* rays, int64_t n, rtg_hit* hits,
                                       int32_t* instance, void* stream) {
    if (!set) return ifail(RTG_INVALID_PARAM, "instance set is NULL");
    if (n < 0) return ifail(RTG_INVALID_PARAM, "negative ray count");
    if (n == 0) return RTG_OK;
    if (!rays || !hits) return ifail(RTG_INVALID_PARAM, "NULL arrays");
    ITRY(cudaSetDevice(set->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : set->scenes[0]->stream;
    float* d_rays = nullptr;
    char* d_out = nullptr;
    const size_t out_bytes = (size_t)n * (sizeof(rtg_hit) + sizeof(int32_t));
    if (cudaMallocAsync(&d_rays, (size_t)n * 32, st) != cudaSuccess ||
        cudaMallocAsync(&d_out, out_bytes, st) != cudaSuccess) {
        if (d_rays) cudaFreeAsync(d_rays, st);
        return ifail(RTG_NO_MEMORY, "instance trace buffers");
    }
    rtg_hit* d_hits = reinterpret_cast<rtg_hit*>(d_out);
    int32_t* d_inst = reinterpret_cast<int32_t*>(d_out + (size_t)n * sizeof(rtg_hit));
    rtg_status rc = RTG_OK;
    if (cudaMemcpyAsync(d_rays, rays, (size_t)n * 32, cudaMemcpyHostToDevice, st) != cudaSuccess)
        rc = ifail(RTG_DEVICE_ERROR, "ray upload");
    if (rc == RTG_OK) rc = trace_instances(set, d_rays, n, d_hits, d_inst, nullptr, 0, 0, st);
    if (rc == RTG_OK && cudaMemcpyAsync(hits, d_hits, (size_t)n * sizeof(rtg_hit), cudaMemcpyDeviceToHost, st) !=
                            cudaSuccess)
        rc = ifail(RTG_DEVICE_ERROR, "hit download");
    if (rc == RTG_OK && instance &&
        cudaMemcpyAsync(instance, d_inst, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        rc = ifail(RTG_DEVICE_ERROR, "instance download");
    cudaFreeAsync(d_rays, st);
    cudaFreeAsync(d_out, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == RTG_OK) rc = ifail(RTG_DEVICE_ERROR, "stream sync");
    return rc;
}

rtg_status rtg_instances_destroy(rtg_instances set) {
    if (!set) return RTG_OK;
    cudaSetDevice(set->device);
    cudaDeviceSynchronize();
    cudaFree(set->d_recs);
    cudaFree(set->d_params);
    cudaFree(set->d_counter);
    delete set;
    return RTG_OK;
}

}  // extern "C"
