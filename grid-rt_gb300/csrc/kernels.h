// kernels.h -- launchers shared by the host API (api.cu) and the kernel files.
#pragma once

#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "common.cuh"

namespace gridrt {

struct BuildArgs {
    const float* verts;
    int64_t nverts;
    const int32_t* idx;
    int64_t ntris;
    int32_t k;
    bool skip_bbox;        // parameters already in `params` (host-resolved)
    GridParams* params;
    BuildWork* work;
    float4* tris;          // 3 per triangle
    float4* wald;          // 3 per triangle: TriAccel records (nullptr: not written)
    int32_t* offsets;      // cell_cap entries
    uint32_t* occ;         // occupancy bitmap, cell_cap words (nullptr: not built)
    int64_t cell_cap;
    int32_t* ids;          // ref_cap entries
    float4* crec;          // optional: 3 x ref_cap float4, triangle records in cell-list order
    int32_t* scratch;      // ref_cap entries
    int64_t ref_cap;
    int64_t* tile_sums;
    int32_t* q_small;
    int32_t* q_med;
    int32_t* q_large;
    int64_t q_small_cap, q_med_cap, q_large_cap;
    int32_t bitmap_words;
    int num_sms;
};

// Cells per tile of the count scan (tile sums: cell capacity / kScanTile + 2).
static constexpr int kScanTile = 1024;

// Process-wide count of kernels launched by this library (diagnostics).
void count_launches(int n);
unsigned long long launches_so_far();

// Side streams and events on which a build runs its three per-cell sorts
// side by side (they touch disjoint cells); nullptr: one after the other.
struct BuildFork {
    cudaStream_t side[2];
    cudaEvent_t fork;
    cudaEvent_t join[2];
    // the triangle-record pass runs on its own stream, beside the whole
    // grid build (it needs only the vertices), joined before the build ends
    cudaStream_t rec;
    cudaEvent_t rec_fork;
    cudaEvent_t rec_clear;   // the offsets and bitmap cleared (the count pass waits for it)
    cudaEvent_t rec_join;
};
void launch_build(const BuildArgs& a, cudaStream_t st, const BuildFork* fork = nullptr);

// Build kernels by work shape (grid sizing per task).
enum BuildKind { BK_BBOX = 0, BK_ZERO, BK_TRI, BK_TILE, BK_SSMALL, BK_SMED, BK_SLARGE, BK_REFS, BK_RECS, kBuildKinds };
// Per-task block counts of every build kernel (the single-scene grid sizes).
void build_blocks(const BuildArgs& a, int sms, int out[kBuildKinds]);
// Batch launch: total[k] blocks for kernel kind k, first[k] a device prefix
// table (ntasks + 1 ints) assigning blocks to tasks.
struct BatchGrid {
    int total[kBuildKinds];
    const int* first[kBuildKinds];
};
void launch_build_batch(const BuildArgs* d_tasks, int ntasks, const BatchGrid& g, int bitmap_words,
                        cudaStream_t st);
// Host resolution of the grid parameters with the C library's powf (used when
// the device flags ST_AMBIGUOUS); defined in api.cu.
void host_resolve(GridParams& p, int32_t k, int64_t ntris, int64_t cell_cap);
// Sets the text rtg_last_error() returns on this thread; defined in api.cu.
void set_last_error(const std::string& msg);
cudaError_t build_setup_attributes(int bitmap_words);

// Read-only view of a built scene for the trace kernels.
struct SceneView {
    const GridParams* params;   // device
    const int32_t* offsets;
    const int32_t* ids;
    const uint32_t* occ;
    const float4* crec;    // records in cell-list order, or nullptr (then ids -> tris)
    const float4* tris;
    const float4* wald;    // TriAccel records: the reported t / u / v of a hit (nullptr: from tris)
};

struct CameraArgs {
    float eye[3], base[3], nu[3], nv[3];
    float inv_w, inv_h;
    int32_t width, height, order;
};

struct TraceCounters {
    unsigned long long rays, cells, tests;
};

// Trace launch shape, chosen per scene (rtg_scene_set_tuning / autotuner).
struct TraceTuning {
    int empty_run = 4;     // empty cells a lane may walk per loop iteration: 2, 4, 8 or 16
    int persistent = 1;    // 1: persistent warps over ray batches; 0: one batch per warp
    int cell_records = 0;  // 1: the build also writes triangle records in cell-list order
    int heavy_cell = 32;   // > 0: rays meeting a list longer than this finish in a warp-per-ray pass
    int heavy_lanes = 32;  // lanes per deferred ray in that pass: 4, 8, 16 or 32
    int refill = -1;       // > 0: idle lanes take new rays once this many are idle (0: finish each batch of 32);
                           // -1 (default): 16 for rays given as arrays, off for camera and frame traces
    int block = 128;       // threads per block of the one-lane trace launch: 64, 128 or 256
    int lanes = 1;         // lanes per ray from the start: 1 (one-lane walk), 2 or 4 (group walk for every ray)
};
// The refill threshold of a launch over camera-generated rays (camera and
// frame traces: coherent, and in a frame each lane's shadow ray follows its
// camera ray, which refill would interleave) or over rays given as arrays.
inline int refill_for(const TraceTuning& t, int mode_is_camera) {
    return t.refill >= 0 ? t.refill : (mode_is_camera ? 0 : 16);
}

// Kernel launch with programmatic stream serialisation when GRIDRT_PDL is on
// (the kernels call pdl_begin() first), a plain launch otherwise.
template <typename... KArgs, typename... Args>
inline void launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                     Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
#if GRIDRT_PDL
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
#endif
    cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Per-launch device state of a single-scene trace: the counters the launch
// zeroes and the deferred-ray and huge-list queues; launches that may overlap
// need distinct slots.
struct TraceSlot {
    unsigned long long* ctr;   // 8 words: ray claims, deferred rays, deferred claims, huge rays, huge claims,
                               // huge entries at the queue's back (lists of kHugeLong+), at its front
    int2* defer;          // {ray, cell} entries
    int32_t defer_cap;
    int2* huge = nullptr; // {ray, cell} entries of rays at a list above kHugeList (nullptr: no block pass)
    int32_t huge_cap = 0;
};
// Lists longer than this are tested by a whole block (the block-per-ray pass)
// when the trace's slot has a huge-list queue.
static constexpr int32_t kHugeList = 2048;
// Huge-list queue entries at lists of at least this many entries are claimed
// first by the block-per-ray pass.
static constexpr int32_t kHugeLong = 8 * kHugeList;

void launch_trace_nearest(const SceneView& s, const float4* rays, int64_t n, int4* hits, TraceCounters* ctr,
                          const TraceSlot& slot, const TraceTuning& tune, int num_sms, cudaStream_t st);
void launch_trace_any(const SceneView& s, const float4* rays, int64_t n, uint8_t* occ, TraceCounters* ctr,
                      const TraceSlot& slot, const TraceTuning& tune, int num_sms, cudaStream_t st);
void launch_trace_camera(const SceneView& s, const CameraArgs& cam, int4* hits, const float* light,
                         float4* shadow_rays, TraceCounters* ctr, const TraceSlot& slot,
                         const TraceTuning& tune, int num_sms, cudaStream_t st, int diffuse = 0,
                         unsigned long long seed = 0);
// Camera rays and, in the same lanes, each hit's shadow ray (MODE_FRAME):
// hits, shadow-ray slots (also the deferred passes' source of shadow rays)
// and occlusion, as launch_trace_camera followed by launch_trace_any over the
// slots.
void launch_trace_frame(const SceneView& s, const CameraArgs& cam, int4* hits, const float* light,
                        float4* shadow_rays, uint8_t* occ, TraceCounters* ctr, const TraceSlot& slot,
                        const TraceTuning& tune, int num_sms, cudaStream_t st);
// Batched tracing: up to kMaxBatchScenes scenes, any number of tasks.
static constexpr int kMaxBatchScenes = 64;
struct BatchScene {
    SceneView view;
};
struct BatchTask {
    long long first;       // start of the task in the flattened, 32-aligned ray space
    long long n;           // rays of the task
    const float4* rays;    // n x 2 float4
    void* out;             // int4 hits (closest) or uint8 occlusion (any)
    int32_t scene;         // index into the scene table
    int32_t mode;          // 0 closest, 1 any
};
void launch_trace_batch(const BatchScene* scenes, int nscenes, const BatchTask* tasks, int ntasks, long long total,
                        const TraceSlot& slot, const TraceTuning& tune, int num_sms, cudaStream_t st);

// Two-level instancing: one entry per instance, in trace order.
struct InstanceRec {
    SceneView view;
    float xf[12];          // local_from_world, 3 x 4 row-major (applied to rays)
    int32_t skip;          // empty or failed grid: never hit
    int32_t pad[3];
};
struct InstanceBox {
    float bmin[3], bmax[3];   // scene box: union of the instances' world boxes
};
// Device bytes of the per-instance grid-parameter table the launcher fills.
size_t instance_params_bytes(int ninst);
// mode 0: closest hit into hits (+ instance index into inst_out when not
// null); mode 1: occlusion into occ.  Launches a parameter-table kernel and
// the trace.
void launch_trace_instances(const InstanceRec* recs, void* d_params, int ninst, const InstanceBox& box,
                            const float4* rays, int64_t n, int4* hits, int32_t* inst_out, uint8_t* occ, int mode,
                            TraceCounters* ctr, unsigned long long* counter, const TraceTuning& tune, int num_sms,
                            cudaStream_t st);

void launch_deform(const float* base, const float* normals, float* out, int64_t nverts, float amp, float freq,
                   float phase, cudaStream_t st);

}  // namespace gridrt
