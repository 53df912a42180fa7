// scene.h -- the scene object behind the rtg_scene handle (internal).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gridrt.h"
#include "common.cuh"
#include "kernels.h"

struct rtg_scene_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int num_sms = 0;

    float* d_verts = nullptr;
    int64_t verts_cap = 0, nverts = 0;   // capacity in floats
    float* d_verts_back = nullptr;       // staged keyframe (rtg_scene_stage_vertices)
    int64_t back_cap = 0, staged_n = 0;
    bool staged = false;
    cudaEvent_t staged_ev = nullptr;     // the staged copy finished
    cudaEvent_t build_ev = nullptr;      // the last build was enqueued up to here
    int32_t* d_idx = nullptr;
    int64_t idx_cap = 0, ntris = 0;      // capacity in ints
    float4* d_tris = nullptr;
    int64_t tris_cap = 0;                // float4 records
    float4* d_wald = nullptr;            // TriAccel records, 3 float4 a triangle
    int64_t wald_cap = 0;

    gridrt::GridParams* d_params = nullptr;
    gridrt::GridParams* h_params = nullptr;      // pinned mirror
    gridrt::BuildWork* d_work = nullptr;
    int32_t* d_offsets = nullptr;
    int64_t cell_cap = 0;
    uint32_t* d_occ = nullptr;
    int64_t occ_cap = 0;
    unsigned long long* d_ray_ctr = nullptr;   // ring of per-launch counters, 8 words a slot
    int2* d_defer = nullptr;                   // ring of per-launch deferred-ray queues (tune.heavy_cell)
    unsigned ctr_seq = 0;
    gridrt::TraceTuning tune;
    int32_t* d_ids = nullptr;
    int64_t ids_cap = 0;
    float4* d_crec = nullptr;            // cell-ordered triangle records (tune.cell_records)
    int64_t crec_cap = 0;                // in float4
    int32_t* d_scratch = nullptr;
    int64_t scratch_cap = 0;
    int64_t* d_tiles = nullptr;
    int64_t tiles_cap = 0;
    int32_t* d_qs = nullptr;
    int64_t qs_cap = 0;
    int32_t* d_qm = nullptr;
    int64_t qm_cap = 0;
    int32_t* d_ql = nullptr;
    int64_t ql_cap = 0;
    int32_t bitmap_words = 32768;

    bool built = false;
    bool crec_built = false;             // the last build wrote cell-ordered records
    int32_t k = 0;
    gridrt::GridParams hp{};   // host copy of the last successful build

    unsigned char* d_io = nullptr;
    int64_t io_cap = 0;
    // rtg_trace_frame_async: shadow-ray area + two output slots, copied back
    // on copy_stream; frame_copied[i] marks the end of slot i's last copy
    unsigned char* d_fring = nullptr;
    int64_t fring_cap = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t frame_traced[2] = {nullptr, nullptr};
    cudaEvent_t frame_copied[2] = {nullptr, nullptr};
    uint64_t frame_seq = 0;              // frames enqueued so far
    // side streams of the build's per-cell sorts (created with the scene)
    gridrt::BuildFork fork{};
    bool have_fork = false;
    gridrt::TraceCounters* d_ctr = nullptr;
};

namespace gridrt {
constexpr unsigned kRayCounters = 32;
constexpr int32_t kDeferCap = 65536;    // deferred rays a launch can queue; more are traced in place
constexpr int32_t kHugeCap = 8192;      // rays a launch can hand to the block-per-ray pass; more stay in the group pass
// deferred-ray queues and huge-list queues of all counter slots, one allocation
constexpr size_t kDeferAlloc = sizeof(int2) * (size_t)kRayCounters * (kDeferCap + kHugeCap);
// Read-only device view of a built scene (for the trace kernels).
SceneView scene_view(rtg_scene s);
// Next per-launch counter slot (and deferred-ray queue) of the scene.
TraceSlot scene_counter(rtg_scene s);
// Camera checks and conversion shared by the camera-ray entry points.
bool camera_ok(const rtg_camera* cam);
CameraArgs camera_args(const rtg_camera* cam);
}  // namespace gridrt
