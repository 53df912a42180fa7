// api.cu -- host side of the C ABI declared in include/gridrt.h.
//
// A scene owns its device buffers (geometry, triangle records, CSR grid,
// build work areas, staging for host-pointer trace calls) and one stream.
// Buffers grow on demand and are never shrunk; capacities carry 1/8 headroom
// so per-frame rebuilds of a deforming mesh do not reallocate.
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gridrt.h"
#include "common.cuh"
#include "kernels.h"

using namespace gridrt;

namespace {

thread_local std::string g_last_error;

rtg_status fail(rtg_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

#define CUDA_TRY(expr)                                                                          \
    do {                                                                                        \
        cudaError_t _e = (expr);                                                                \
        if (_e != cudaSuccess) {                                                                \
            return fail(_e == cudaErrorMemoryAllocation ? RTG_NO_MEMORY : RTG_DEVICE_ERROR,     \
                        std::string(#expr) + ": " + cudaGetErrorString(_e));                    \
        }                                                                                       \
    } while (0)

template <class T>
cudaError_t grow(T*& p, int64_t& cap, int64_t need) {
    if (need <= cap && p) return cudaSuccess;
    int64_t n = need + need / 8 + 64;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc((void**)&p, (size_t)n * sizeof(T));
    if (e == cudaSuccess) cap = n;
    return e;
}

}  // namespace

#include "scene.h"

namespace {

rtg_status set_device(rtg_scene s) {
    CUDA_TRY(cudaSetDevice(s->device));
    return RTG_OK;
}

int64_t ref_capacity(const rtg_scene s) {
    int64_t c = s->ids_cap < s->scratch_cap ? s->ids_cap : s->scratch_cap;
    if (s->tune.cell_records) c = c < s->crec_cap / 3 ? c : s->crec_cap / 3;
    return c;
}


rtg_status ensure_grid_buffers(rtg_scene s, int64_t cells_plus_one, int64_t refs) {
    CUDA_TRY(grow(s->d_offsets, s->cell_cap, cells_plus_one));
    CUDA_TRY(grow(s->d_occ, s->occ_cap, s->cell_cap));
    CUDA_TRY(grow(s->d_tiles, s->tiles_cap, s->cell_cap / kScanTile + 2));
    CUDA_TRY(grow(s->d_ids, s->ids_cap, refs));
    CUDA_TRY(grow(s->d_scratch, s->scratch_cap, refs));
    if (s->tune.cell_records) CUDA_TRY(grow(s->d_crec, s->crec_cap, 3 * s->ids_cap));
    const int64_t R = ref_capacity(s);
    CUDA_TRY(grow(s->d_qs, s->qs_cap, R / 2 + 2));
    CUDA_TRY(grow(s->d_qm, s->qm_cap, R / 33 + 2));
    CUDA_TRY(grow(s->d_ql, s->ql_cap, R / (SORT_MED_MAX + 1) + 2));
    return RTG_OK;
}

// Cell-ordered records enabled after the id buffers were sized: give the
// record buffer the same capacity before the next build.
rtg_status ensure_cell_records(rtg_scene s) {
    const int64_t raw = s->ids_cap < s->scratch_cap ? s->ids_cap : s->scratch_cap;
    if (!s->tune.cell_records || !s->d_offsets || s->crec_cap >= 3 * raw) return RTG_OK;
    return ensure_grid_buffers(s, s->cell_cap, raw);
}

// A staged keyframe becomes the build's vertices: the build stream waits for
// its copy and the two vertex buffers swap.
rtg_status apply_staged(rtg_scene s, cudaStream_t st) {
    if (!s->staged) return RTG_OK;
    CUDA_TRY(cudaStreamWaitEvent(st, s->staged_ev, 0));
    std::swap(s->d_verts, s->d_verts_back);
    std::swap(s->verts_cap, s->back_cap);
    s->staged = false;
    return RTG_OK;
}

// Marks the end of the builds enqueued so far, for the next staged copy.
void mark_build(rtg_scene s, cudaStream_t st) {
    if (s->build_ev) cudaEventRecord(s->build_ev, st);
}

BuildArgs make_args(rtg_scene s, int32_t k, bool skip_bbox) {
    BuildArgs a{};   // zeroed padding: batches compare argument blocks bytewise
    a.verts = s->d_verts;
    a.nverts = s->nverts;
    a.idx = s->d_idx;
    a.ntris = s->ntris;
    a.k = k;
    a.skip_bbox = skip_bbox;
    a.params = s->d_params;
    a.work = s->d_work;
    a.tris = s->d_tris;
    a.wald = s->d_wald;
    a.offsets = s->d_offsets;
    a.occ = s->d_occ;
    a.cell_cap = s->cell_cap < s->occ_cap ? s->cell_cap : s->occ_cap;
    a.ids = s->d_ids;
    a.crec = s->tune.cell_records ? s->d_crec : nullptr;
    a.scratch = s->d_scratch;
    a.ref_cap = ref_capacity(s);
    a.tile_sums = s->d_tiles;
    a.q_small = s->d_qs;
    a.q_med = s->d_qm;
    a.q_large = s->d_ql;
    a.q_small_cap = s->qs_cap;
    a.q_med_cap = s->qm_cap;
    a.q_large_cap = s->ql_cap;
    a.bitmap_words = s->bitmap_words;
    a.num_sms = s->num_sms;
    return a;
}

// Host resolution of the grid parameters with the C library's powf, used when
// the device flagged that the last ulp of powf decides a cell count.  Same
// float operation order as src/rtplugins/UniformGridAccStructBuilder.cpp:86-98
// and src/rtplugins/UniformGridAccStruct.cpp:56-62 (compiled without FMA
// contraction).
}  // namespace

namespace gridrt {
void set_last_error(const std::string& msg) { g_last_error = msg; }

void host_resolve(GridParams& p, int32_t k, int64_t ntris, int64_t cell_cap) {
    volatile float diag[3];
    for (int d = 0; d < 3; ++d) diag[d] = p.bmax[d] - p.bmin[d];
    volatile float v01 = diag[0] * diag[1];
    volatile float V = v01 * diag[2];
    const int32_t kn = (int32_t)((uint32_t)k * (uint32_t)ntris);
    volatile float q = (float)kn / V;
    volatile float factor = powf(q, 1.0f / 3.0f);
    int64_t nc = 1;
    uint32_t st = 0;
    for (int d = 0; d < 3; ++d) {
        volatile float m = diag[d] * factor;
        float c = ceilf(m);
        int32_t r = (c >= 1.0f && c < 2147483648.0f) ? (int32_t)c : 0;
        if (r <= 0) st |= ST_TOO_BIG;
        p.res[d] = r;
        nc *= (r > 0 ? r : 1);
    }
    for (int d = 0; d < 3; ++d) {
        volatile float ext = p.bmax[d] - p.bmin[d];
        volatile float cs = ext / (float)(p.res[d] > 0 ? p.res[d] : 1);
        p.cell[d] = cs;
        p.inv[d] = 1.0f / cs;
    }
    if (nc >= INT32_MAX) st |= ST_TOO_BIG;
    if (nc + 1 > cell_cap) st |= ST_CELL_CAP;
    p.ncells = nc;
    p.nrefs = 0;
    p.k = k;
    p.ntris = ntris;
    p.status = st;
    p.max_list = 0u;
}
}  // namespace gridrt

namespace {

rtg_status read_params(rtg_scene s) {
    CUDA_TRY(cudaMemcpyAsync(s->h_params, s->d_params, sizeof(GridParams), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return RTG_OK;
}

rtg_status read_clear_sticky(rtg_scene s, uint32_t* out) {
    char* addr = reinterpret_cast<char*>(s->d_work) + offsetof(BuildWork, sticky);
    CUDA_TRY(cudaMemcpyAsync(out, addr, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaMemsetAsync(addr, 0, sizeof(uint32_t), s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return RTG_OK;
}

rtg_status enqueue_build(rtg_scene s, int32_t k, bool skip_bbox, cudaStream_t st) {
    if (skip_bbox)
        CUDA_TRY(cudaMemsetAsync(reinterpret_cast<char*>(s->d_work) + offsetof(BuildWork, nsort), 0,
                                 sizeof(BuildWork::nsort), st));
    launch_build(make_args(s, k, skip_bbox), st, s->have_fork ? &s->fork : nullptr);
    CUDA_TRY(cudaGetLastError());
    return RTG_OK;
}

rtg_status empty_grid(rtg_scene s, int32_t k) {
    std::memset(&s->hp, 0, sizeof(GridParams));
    s->hp.k = k;
    s->built = true;
    s->k = k;
    return RTG_OK;
}

cudaStream_t pick(rtg_scene s, void* stream) { return stream ? (cudaStream_t)stream : s->stream; }

}  // namespace

namespace gridrt {
// Each trace launch takes the next of kRayCounters counter slots (and the
// deferred-ray queue beside it), so up to that many launches may be in
// flight at once.
TraceSlot scene_counter(rtg_scene s) {
    const unsigned slot = __atomic_fetch_add(&s->ctr_seq, 1u, __ATOMIC_RELAXED) % kRayCounters;
    TraceSlot t;
    t.ctr = s->d_ray_ctr + 8 * (size_t)slot;
    t.defer = s->d_defer ? s->d_defer + (size_t)slot * kDeferCap : nullptr;
    t.defer_cap = s->d_defer ? kDeferCap : 0;
    // the block-per-ray pass is launched for scenes whose last checked build
    // had a list above kHugeList (the group pass handles such lists anyway)
    if (s->d_defer && s->hp.max_list > (uint32_t)kHugeList) {
        t.huge = s->d_defer + (size_t)kRayCounters * kDeferCap + (size_t)slot * kHugeCap;
        t.huge_cap = kHugeCap;
    }
    return t;
}
}  // namespace gridrt

namespace {
TraceSlot next_counter(rtg_scene s) { return scene_counter(s); }

}  // namespace

namespace gridrt {
SceneView scene_view(rtg_scene s) {
    SceneView v;
    v.params = s->d_params;
    v.offsets = s->d_offsets;
    v.ids = s->d_ids;
    v.occ = s->d_occ;
    v.crec = (s->tune.cell_records && s->crec_built) ? s->d_crec : nullptr;
    v.tris = s->d_tris;
    v.wald = s->d_wald;
    return v;
}
}  // namespace gridrt

namespace {
SceneView view(rtg_scene s) { return scene_view(s); }

rtg_status ensure_io(rtg_scene s, int64_t bytes) {
    if (bytes <= s->io_cap && s->d_io) return RTG_OK;
    CUDA_TRY(grow(s->d_io, s->io_cap, bytes));
    return RTG_OK;
}

}  // namespace

extern "C" {

const char* rtg_version(void) { return "gridrt 0.1 (sm_103a)"; }
const char* rtg_last_error(void) { return g_last_error.c_str(); }

rtg_status rtg_scene_create(int device, void* stream, rtg_scene* out) {
    if (!out) return fail(RTG_INVALID_PARAM, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(RTG_INVALID_PARAM, "no such device");
    CUDA_TRY(cudaSetDevice(device));
    rtg_scene s = new rtg_scene_s();
    s->device = device;
    cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (stream) {
        s->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete s;
            return fail(RTG_DEVICE_ERROR, "stream creation failed");
        }
        s->own_stream = true;
    }
    int max_optin = 0;
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    // bitmap for the large-cell sort: up to 128 KiB (1M triangle ids per pass)
    int words = 32768;
    while (words * 4 + 4096 > max_optin && words > 1024) words >>= 1;
    s->bitmap_words = words;
    rtg_status rc = RTG_OK;
    if (build_setup_attributes(words) != cudaSuccess) rc = fail(RTG_DEVICE_ERROR, "smem attribute");
    if (rc == RTG_OK && cudaMalloc(&s->d_params, sizeof(GridParams)) != cudaSuccess) rc = fail(RTG_NO_MEMORY, "params");
    if (rc == RTG_OK && cudaMallocHost(&s->h_params, sizeof(GridParams)) != cudaSuccess) rc = fail(RTG_NO_MEMORY, "pinned");
    if (rc == RTG_OK && cudaMalloc(&s->d_work, sizeof(BuildWork)) != cudaSuccess) rc = fail(RTG_NO_MEMORY, "work");
    if (rc == RTG_OK && cudaMalloc(&s->d_ctr, sizeof(TraceCounters)) != cudaSuccess) rc = fail(RTG_NO_MEMORY, "ctr");
    if (rc == RTG_OK && cudaMalloc(&s->d_ray_ctr, 8 * kRayCounters * sizeof(unsigned long long)) != cudaSuccess)
        rc = fail(RTG_NO_MEMORY, "ray counters");
    if (rc == RTG_OK && s->tune.heavy_cell > 0 &&
        cudaMalloc(&s->d_defer, kDeferAlloc) != cudaSuccess) {
        s->d_defer = nullptr;
        rc = fail(RTG_NO_MEMORY, "deferred-ray queues");
    }
    if (rc == RTG_OK) {
        // the sorts' side streams; without them the build stays on one stream
        bool ok = cudaStreamCreateWithFlags(&s->fork.side[0], cudaStreamNonBlocking) == cudaSuccess;
        ok = ok && cudaStreamCreateWithFlags(&s->fork.side[1], cudaStreamNonBlocking) == cudaSuccess;
        ok = ok && cudaEventCreateWithFlags(&s->fork.fork, cudaEventDisableTiming) == cudaSuccess;
        ok = ok && cudaEventCreateWithFlags(&s->fork.join[0], cudaEventDisableTiming) == cudaSuccess;
        ok = ok && cudaEventCreateWithFlags(&s->fork.join[1], cudaEventDisableTiming) == cudaSuccess;
        ok = ok && cudaStreamCreateWithFlags(&s->fork.rec, cudaStreamNonBlocking) == cudaSuccess;
        ok = ok && cudaEventCreateWithFlags(&s->fork.rec_fork, cudaEventDisableTiming) == cudaSuccess;
        ok = ok && cudaEventCreateWithFlags(&s->fork.rec_clear, cudaEventDisableTiming) == cudaSuccess;
        ok = ok && cudaEventCreateWithFlags(&s->fork.rec_join, cudaEventDisableTiming) == cudaSuccess;
        s->have_fork = ok;
        if (!ok) cudaGetLastError();
    }
    if (rc == RTG_OK) {
        BuildWork w;
        std::memset(&w, 0, sizeof(w));
        for (int d = 0; d < 3; ++d) { w.keys[d] = 0xffffffffu; w.keys[3 + d] = 0u; }
        cudaMemcpy(s->d_work, &w, sizeof(w), cudaMemcpyHostToDevice);
        cudaMemset(s->d_ctr, 0, sizeof(TraceCounters));
        cudaMemset(s->d_params, 0, sizeof(GridParams));
        if (cudaGetLastError() != cudaSuccess) rc = fail(RTG_DEVICE_ERROR, "init copies");
    }
    if (rc != RTG_OK) {
        rtg_scene_destroy(s);
        return rc;
    }
    *out = s;
    return RTG_OK;
}

rtg_status rtg_scene_destroy(rtg_scene s) {
    if (!s) return RTG_OK;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    cudaFree(s->d_verts);
    cudaFree(s->d_idx);
    cudaFree(s->d_tris);
    cudaFree(s->d_wald);
    cudaFree(s->d_params);
    if (s->h_params) cudaFreeHost(s->h_params);
    cudaFree(s->d_work);
    cudaFree(s->d_offsets);
    cudaFree(s->d_occ);
    cudaFree(s->d_ray_ctr);
    cudaFree(s->d_defer);
    cudaFree(s->d_ids);
    cudaFree(s->d_scratch);
    cudaFree(s->d_crec);
    cudaFree(s->d_tiles);
    cudaFree(s->d_qs);
    cudaFree(s->d_qm);
    cudaFree(s->d_ql);
    cudaFree(s->d_io);
    cudaFree(s->d_ctr);
    cudaFree(s->d_verts_back);
    if (s->copy_stream) cudaStreamSynchronize(s->copy_stream);
    for (int i = 0; i < 2; ++i) {
        if (s->fork.side[i]) {
            cudaStreamSynchronize(s->fork.side[i]);
            cudaStreamDestroy(s->fork.side[i]);
        }
        if (s->fork.join[i]) cudaEventDestroy(s->fork.join[i]);
    }
    if (s->fork.fork) cudaEventDestroy(s->fork.fork);
    if (s->fork.rec) {
        cudaStreamSynchronize(s->fork.rec);
        cudaStreamDestroy(s->fork.rec);
    }
    if (s->fork.rec_fork) cudaEventDestroy(s->fork.rec_fork);
    if (s->fork.rec_clear) cudaEventDestroy(s->fork.rec_clear);
    if (s->fork.rec_join) cudaEventDestroy(s->fork.rec_join);
    cudaFree(s->d_fring);
    for (int i = 0; i < 2; ++i) {
        if (s->frame_traced[i]) cudaEventDestroy(s->frame_traced[i]);
        if (s->frame_copied[i]) cudaEventDestroy(s->frame_copied[i]);
    }
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    if (s->staged_ev) cudaEventDestroy(s->staged_ev);
    if (s->build_ev) cudaEventDestroy(s->build_ev);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return RTG_OK;
}

rtg_status rtg_scene_stream(rtg_scene s, void** stream_out) {
    if (!s || !stream_out) return fail(RTG_INVALID_PARAM, "NULL argument");
    *stream_out = (void*)s->stream;
    return RTG_OK;
}

static rtg_status set_geometry(rtg_scene s, const float* verts, int64_t nverts, const int32_t* tris, int64_t ntris,
                               cudaMemcpyKind kind, cudaStream_t st) {
    if (!s) return fail(RTG_INVALID_PARAM, "scene is NULL");
    if (nverts < 0 || ntris < 0 || (nverts > 0 && !verts) || (ntris > 0 && !tris))
        return fail(RTG_INVALID_PARAM, "bad geometry arrays");
    if (ntris > (int64_t)INT32_MAX / 8 || nverts > (int64_t)INT32_MAX)
        return fail(RTG_INVALID_PARAM, "geometry larger than the int32 index space");
    rtg_status rc = set_device(s);
    if (rc) return rc;
    if (s->staged) {   // a staged keyframe of the old geometry is dropped
        CUDA_TRY(cudaStreamWaitEvent(st, s->staged_ev, 0));
        s->staged = false;
    }
    CUDA_TRY(grow(s->d_verts, s->verts_cap, 3 * nverts + 4));
    CUDA_TRY(grow(s->d_idx, s->idx_cap, 3 * ntris + 4));
    CUDA_TRY(grow(s->d_tris, s->tris_cap, 3 * ntris + 3));
    CUDA_TRY(grow(s->d_wald, s->wald_cap, 3 * ntris + 3));
    if (nverts) CUDA_TRY(cudaMemcpyAsync(s->d_verts, verts, sizeof(float) * 3 * nverts, kind, st));
    if (ntris) CUDA_TRY(cudaMemcpyAsync(s->d_idx, tris, sizeof(int32_t) * 3 * ntris, kind, st));
    s->nverts = nverts;
    s->ntris = ntris;
    s->built = false;
    if (st != s->stream) CUDA_TRY(cudaStreamSynchronize(st));
    return RTG_OK;
}

rtg_status rtg_scene_set_geometry(rtg_scene s, const float* verts, int64_t nverts, const int32_t* tris, int64_t ntris,
                                  void* stream) {
    if (!s) return fail(RTG_INVALID_PARAM, "scene is NULL");
    cudaStream_t st = pick(s, stream);
    rtg_status rc = set_geometry(s, verts, nverts, tris, ntris, cudaMemcpyHostToDevice, st);
    if (rc) return rc;
    CUDA_TRY(cudaStreamSynchronize(st));
    return RTG_OK;
}

rtg_status rtg_scene_set_geometry_device(rtg_scene s, const float* d_verts, int64_t nverts, const int32_t* d_tris,
                                         int64_t ntris, void* stream) {
    if (!s) return fail(RTG_INVALID_PARAM, "scene is NULL");
    return set_geometry(s, d_verts, nverts, d_tris, ntris, cudaMemcpyDeviceToDevice, pick(s, stream));
}

rtg_status rtg_scene_update_vertices(rtg_scene s, const float* verts, int64_t nverts, int from_device, void* stream) {
    if (!s || (!verts && nverts)) return fail(RTG_INVALID_PARAM, "NULL argument");
    if (nverts != s->nverts) return fail(RTG_INVALID_PARAM, "vertex count differs from the scene's");
    rtg_status rc = set_device(s);
    if (rc) return rc;
    cudaStream_t st = pick(s, stream);
    if (nverts)
        CUDA_TRY(cudaMemcpyAsync(s->d_verts, verts, sizeof(float) * 3 * nverts,
                                 from_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
    s->built = false;
    return RTG_OK;
}

rtg_status rtg_scene_stage_vertices(rtg_scene s, const float* h_verts, int64_t nverts, void* copy_stream) {
    if (!s || (!h_verts && nverts)) return fail(RTG_INVALID_PARAM, "NULL argument");
    if (nverts != s->nverts) return fail(RTG_INVALID_PARAM, "vertex count differs from the scene's");
    rtg_status rc = set_device(s);
    if (rc) return rc;
    if (!s->staged_ev) {
        CUDA_TRY(cudaEventCreateWithFlags(&s->staged_ev, cudaEventDisableTiming));
        CUDA_TRY(cudaEventCreateWithFlags(&s->build_ev, cudaEventDisableTiming));
    }
    CUDA_TRY(grow(s->d_verts_back, s->back_cap, 3 * nverts));
    cudaStream_t cs = copy_stream ? (cudaStream_t)copy_stream : s->stream;
    // the back buffer was last read by a build enqueued before the last one
    // marked; an unconsumed earlier stage may still be copying into it
    CUDA_TRY(cudaStreamWaitEvent(cs, s->build_ev, 0));
    if (s->staged) CUDA_TRY(cudaStreamWaitEvent(cs, s->staged_ev, 0));
    if (nverts)
        CUDA_TRY(cudaMemcpyAsync(s->d_verts_back, h_verts, sizeof(float) * 3 * nverts, cudaMemcpyHostToDevice, cs));
    CUDA_TRY(cudaEventRecord(s->staged_ev, cs));
    s->staged = true;   // the current grid stays traceable until the next build
    return RTG_OK;
}

rtg_status rtg_scene_deform_vertices(rtg_scene s, const float* d_base, const float* d_normals, float amp, float freq,
                                     float phase, void* stream) {
    if (!s || !d_base || !d_normals) return fail(RTG_INVALID_PARAM, "NULL argument");
    rtg_status rc = set_device(s);
    if (rc) return rc;
    launch_deform(d_base, d_normals, s->d_verts, s->nverts, amp, freq, phase, pick(s, stream));
    CUDA_TRY(cudaGetLastError());
    s->built = false;
    return RTG_OK;
}

rtg_status rtg_scene_reserve(rtg_scene s, int64_t ncells, int64_t nrefs) {
    if (!s || ncells < 0 || nrefs < 0) return fail(RTG_INVALID_PARAM, "bad reserve");
    rtg_status rc = set_device(s);
    if (rc) return rc;
    return ensure_grid_buffers(s, ncells + 1, nrefs);
}

rtg_status rtg_scene_build_async(rtg_scene s, int32_t k, void* stream) {
    if (!s) return fail(RTG_INVALID_PARAM, "scene is NULL");
    if (k <= 0) return fail(RTG_INVALID_PARAM, "k must be positive");
    rtg_status rc = set_device(s);
    if (rc) return rc;
    s->k = k;
    if (s->ntris == 0 || s->nverts == 0) return empty_grid(s, k);
    // The first build of a scene runs synchronously: it sizes the buffers.
    if (!s->d_offsets || s->hp.ncells == 0) return rtg_scene_build(s, k, stream);
    rc = ensure_cell_records(s);
    if (rc) return rc;
    rc = apply_staged(s, pick(s, stream));
    if (rc) return rc;
    rc = enqueue_build(s, k, false, pick(s, stream));
    if (rc) return rc;
    mark_build(s, pick(s, stream));
    // Trace calls may follow on the same stream: the trace kernels read the
    // device-side status and return misses if this build failed, and
    // rtg_scene_build_check reports the failure.
    s->built = true;
    s->crec_built = s->tune.cell_records != 0;
    return RTG_OK;
}

rtg_status rtg_scene_build_check(rtg_scene s, void* stream) {
    if (!s) return fail(RTG_INVALID_PARAM, "scene is NULL");
    if (s->ntris == 0 || s->nverts == 0) return s->built ? RTG_OK : fail(RTG_NOT_BUILT, "not built");
    rtg_status rc = set_device(s);
    if (rc) return rc;
    CUDA_TRY(cudaStreamSynchronize(pick(s, stream)));
    rc = read_params(s);
    if (rc) return rc;
    uint32_t sticky = 0;
    rc = read_clear_sticky(s, &sticky);
    if (rc) return rc;
    const uint32_t st = s->h_params->status | sticky;
    if (st & (ST_CELL_CAP | ST_REF_CAP | ST_SORT_CAP | ST_AMBIGUOUS))
        return fail(RTG_NO_MEMORY, "asynchronous build needs a synchronous rebuild (capacity or resolution)");
    if (st & ST_TOO_BIG) return fail(RTG_INVALID_PARAM, "grid exceeds the int32 index space");
    if (st & ST_BAD_RANGE) return fail(RTG_INVALID_GEOMETRY, "non-finite vertex or triangle outside the grid");
    s->hp = *s->h_params;
    s->built = true;
    return RTG_OK;
}

rtg_status rtg_scene_build(rtg_scene s, int32_t k, void* stream) {
    if (!s) return fail(RTG_INVALID_PARAM, "scene is NULL");
    if (k <= 0) return fail(RTG_INVALID_PARAM, "k must be positive");
    rtg_status rc = set_device(s);
    if (rc) return rc;
    cudaStream_t st = pick(s, stream);
    if (st != s->stream) {
        // keep the scene's own stream ordered behind the caller's
        CUDA_TRY(cudaStreamSynchronize(st));
    }
    s->k = k;
    if (s->ntris == 0 || s->nverts == 0) return empty_grid(s, k);
    if (!s->d_offsets) {
        rc = ensure_grid_buffers(s, 1, 1);
        if (rc) return rc;
    }
    rc = ensure_cell_records(s);
    if (rc) return rc;
    rc = apply_staged(s, s->stream);
    if (rc) return rc;
    s->built = false;
    bool skip_bbox = false;
    for (int attempt = 0; attempt < 6; ++attempt) {
        rc = enqueue_build(s, k, skip_bbox, s->stream);
        if (rc) return rc;
        rc = read_params(s);
        if (rc) return rc;
        GridParams p = *s->h_params;
        if (p.status & ST_TOO_BIG) return fail(RTG_INVALID_PARAM, "grid exceeds the int32 index space");
        if (p.status & ST_AMBIGUOUS) {
            host_resolve(p, k, s->ntris, s->cell_cap);
            if (p.status & ST_TOO_BIG) return fail(RTG_INVALID_PARAM, "grid exceeds the int32 index space");
            if (p.status & ST_CELL_CAP) {
                rc = ensure_grid_buffers(s, p.ncells + 1, ref_capacity(s));
                if (rc) return rc;
                p.status &= ~ST_CELL_CAP;
            }
            CUDA_TRY(cudaMemcpyAsync(s->d_params, &p, sizeof(GridParams), cudaMemcpyHostToDevice, s->stream));
            skip_bbox = true;
            continue;
        }
        if (p.status & ST_CELL_CAP) {
            const int64_t guess = ref_capacity(s) > 8 * s->ntris ? ref_capacity(s) : 8 * s->ntris;
            rc = ensure_grid_buffers(s, p.ncells + 1, guess);
            if (rc) return rc;
            skip_bbox = false;
            continue;
        }
        if (p.status & (ST_REF_CAP | ST_SORT_CAP)) {
            rc = ensure_grid_buffers(s, s->cell_cap, p.nrefs);
            if (rc) return rc;
            skip_bbox = false;
            continue;
        }
        if (p.status & ST_BAD_RANGE)
            return fail(RTG_INVALID_GEOMETRY, "non-finite vertex or triangle outside the grid");
        s->hp = p;
        s->built = true;
        s->crec_built = s->tune.cell_records != 0;
        mark_build(s, s->stream);
        uint32_t sticky = 0;
        return read_clear_sticky(s, &sticky);   // earlier attempts of this call are resolved
    }
    return fail(RTG_DEVICE_ERROR, "grid build did not converge");
}

rtg_status rtg_scene_grid_info(rtg_scene s, rtg_grid_info* out) {
    if (!s || !out) return fail(RTG_INVALID_PARAM, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    const GridParams& p = s->hp;
    for (int d = 0; d < 3; ++d) {
        out->res[d] = p.res[d];
        out->bmin[d] = p.bmin[d];
        out->bmax[d] = p.bmax[d];
        out->cell[d] = p.cell[d];
        out->inv_cell[d] = p.inv[d];
    }
    out->ncells = p.ncells;
    out->nrefs = p.nrefs;
    out->k = s->k;
    out->built = s->built ? 1 : 0;
    return RTG_OK;
}

rtg_status rtg_scene_grid_download(rtg_scene s, int32_t* offsets, int32_t* ids) {
    if (!s || !offsets) return fail(RTG_INVALID_PARAM, "NULL argument");
    if (!s->built) return fail(RTG_NOT_BUILT, "scene not built");
    rtg_status rc = set_device(s);
    if (rc) return rc;
    if (s->hp.ncells == 0) {
        offsets[0] = 0;
        return RTG_OK;
    }
    CUDA_TRY(cudaMemcpyAsync(offsets, s->d_offsets, sizeof(int32_t) * (s->hp.ncells + 1), cudaMemcpyDeviceToHost,
                             s->stream));
    if (s->hp.nrefs && ids)
        CUDA_TRY(cudaMemcpyAsync(ids, s->d_ids, sizeof(int32_t) * s->hp.nrefs, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return RTG_OK;
}

rtg_status rtg_scene_download_vertices(rtg_scene s, float* verts) {
    if (!s || (!verts && s->nverts)) return fail(RTG_INVALID_PARAM, "NULL argument");
    rtg_status rc = set_device(s);
    if (rc) return rc;
    if (s->nverts)
        CUDA_TRY(cudaMemcpyAsync(verts, s->d_verts, sizeof(float) * 3 * s->nverts, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return RTG_OK;
}

rtg_status rtg_scene_grid_device(rtg_scene s, const int32_t** d_offsets, const int32_t** d_ids, const float** d_tris) {
    if (!s) return fail(RTG_INVALID_PARAM, "scene is NULL");
    if (d_offsets) *d_offsets = s->d_offsets;
    if (d_ids) *d_ids = s->d_ids;
    if (d_tris) *d_tris = reinterpret_cast<const float*>(s->d_tris);
    return RTG_OK;
}

static rtg_status check_traceable(rtg_scene s, int64_t n) {
    if (!s) return fail(RTG_INVALID_PARAM, "scene is NULL");
    if (n < 0) return fail(RTG_INVALID_PARAM, "negative ray count");
    if (!s->built) return fail(RTG_NOT_BUILT, "scene not built");
    return set_device(s);
}

rtg_status rtg_trace_nearest_device(rtg_scene s, const float* d_rays, int64_t n, rtg_hit* d_hits, int32_t flags,
                                    void* stream) {
    rtg_status rc = check_traceable(s, n);
    if (rc) return rc;
    if (n == 0) return RTG_OK;
    if (!d_rays || !d_hits) return fail(RTG_INVALID_PARAM, "NULL arrays");
    cudaStream_t st = pick(s, stream);
    if (s->hp.ncells == 0) {
        CUDA_TRY(cudaMemsetAsync(d_hits, 0xff, sizeof(rtg_hit) * n, st));   // id = -1 (t/u/v NaN-bit pattern)
        return RTG_OK;
    }
    launch_trace_nearest(view(s), reinterpret_cast<const float4*>(d_rays), n, reinterpret_cast<int4*>(d_hits),
                         (flags & RTG_TRACE_COUNTERS) ? s->d_ctr : nullptr, next_counter(s), s->tune, s->num_sms, st);
    CUDA_TRY(cudaGetLastError());
    return RTG_OK;
}

rtg_status rtg_trace_any_device(rtg_scene s, const float* d_rays, int64_t n, uint8_t* d_occ, int32_t flags,
                                void* stream) {
    rtg_status rc = check_traceable(s, n);
    if (rc) return rc;
    if (n == 0) return RTG_OK;
    if (!d_rays || !d_occ) return fail(RTG_INVALID_PARAM, "NULL arrays");
    cudaStream_t st = pick(s, stream);
    if (s->hp.ncells == 0) {
        CUDA_TRY(cudaMemsetAsync(d_occ, 0, n, st));
        return RTG_OK;
    }
    launch_trace_any(view(s), reinterpret_cast<const float4*>(d_rays), n, d_occ,
                     (flags & RTG_TRACE_COUNTERS) ? s->d_ctr : nullptr, next_counter(s), s->tune, s->num_sms, st);
    CUDA_TRY(cudaGetLastError());
    return RTG_OK;
}

rtg_status rtg_trace_nearest(rtg_scene s, const float* rays, int64_t n, rtg_hit* hits, int32_t flags, void* stream) {
    rtg_status rc = check_traceable(s, n);
    if (rc) return rc;
    if (n == 0) return RTG_OK;
    if (!rays || !hits) return fail(RTG_INVALID_PARAM, "NULL arrays");
    cudaStream_t st = pick(s, stream);
    rc = ensure_io(s, n * 48);
    if (rc) return rc;
    float* d_rays = reinterpret_cast<float*>(s->d_io);
    rtg_hit* d_hits = reinterpret_cast<rtg_hit*>(s->d_io + n * 32);
    CUDA_TRY(cudaMemcpyAsync(d_rays, rays, n * 32, cudaMemcpyHostToDevice, st));
    rc = rtg_trace_nearest_device(s, d_rays, n, d_hits, flags, st);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(hits, d_hits, n * 16, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return RTG_OK;
}

rtg_status rtg_trace_any(rtg_scene s, const float* rays, int64_t n, uint8_t* occ, int32_t flags, void* stream) {
    rtg_status rc = check_traceable(s, n);
    if (rc) return rc;
    if (n == 0) return RTG_OK;
    if (!rays || !occ) return fail(RTG_INVALID_PARAM, "NULL arrays");
    cudaStream_t st = pick(s, stream);
    rc = ensure_io(s, n * 33 + 16);
    if (rc) return rc;
    float* d_rays = reinterpret_cast<float*>(s->d_io);
    uint8_t* d_occ = s->d_io + n * 32;
    CUDA_TRY(cudaMemcpyAsync(d_rays, rays, n * 32, cudaMemcpyHostToDevice, st));
    rc = rtg_trace_any_device(s, d_rays, n, d_occ, flags, st);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(occ, d_occ, n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return RTG_OK;
}

}  // extern "C"

namespace gridrt {
bool camera_ok(const rtg_camera* cam) {
    if (!cam || cam->width <= 0 || cam->height <= 0) return false;
    if ((int64_t)cam->width * cam->height > ((int64_t)1 << 31)) return false;
    if (cam->order == RTG_ORDER_MORTON8 && ((cam->width & 7) || (cam->height & 7))) return false;
    return cam->order == RTG_ORDER_SCANLINE || cam->order == RTG_ORDER_MORTON8;
}

CameraArgs camera_args(const rtg_camera* cam) {
    CameraArgs c;
    for (int a = 0; a < 3; ++a) {
        c.eye[a] = cam->eye[a];
        c.base[a] = cam->base_dir[a];
        c.nu[a] = cam->near_u[a];
        c.nv[a] = cam->near_v[a];
    }
    // PinholeCamera::newFrame: _invWidth = 1.0f / _screenWidth (src/rtplugins/PinholeCamera.cpp:52-53)
    volatile float w = (float)cam->width, h = (float)cam->height;
    c.inv_w = 1.0f / w;
    c.inv_h = 1.0f / h;
    c.width = cam->width;
    c.height = cam->height;
    c.order = cam->order;
    return c;
}
}  // namespace gridrt

extern "C" {

rtg_status rtg_trace_camera_device(rtg_scene s, const rtg_camera* cam, rtg_hit* d_hits, const float* light_pos,
                                   float* d_shadow_rays, int32_t flags, void* stream) {
    rtg_status rc = check_traceable(s, 0);
    if (rc) return rc;
    if (!camera_ok(cam)) return fail(RTG_INVALID_PARAM, "bad camera (size, or Morton order needs multiples of 8)");
    if (!d_hits) return fail(RTG_INVALID_PARAM, "NULL hits");
    cudaStream_t st = pick(s, stream);
    const int64_t n = (int64_t)cam->width * cam->height;
    if (s->hp.ncells == 0) {
        CUDA_TRY(cudaMemsetAsync(d_hits, 0xff, sizeof(rtg_hit) * n, st));
        if (d_shadow_rays) CUDA_TRY(cudaMemsetAsync(d_shadow_rays, 0xff, 32 * n, st));
        return RTG_OK;
    }
    launch_trace_camera(view(s), camera_args(cam), reinterpret_cast<int4*>(d_hits), light_pos,
                        reinterpret_cast<float4*>(d_shadow_rays), (flags & RTG_TRACE_COUNTERS) ? s->d_ctr : nullptr,
                        next_counter(s), s->tune, s->num_sms, st);
    CUDA_TRY(cudaGetLastError());
    return RTG_OK;
}

rtg_status rtg_trace_camera_diffuse_device(rtg_scene s, const rtg_camera* cam, uint64_t seed, rtg_hit* d_hits,
                                           float* d_secondary_rays, int32_t flags, void* stream) {
    rtg_status rc = check_traceable(s, 0);
    if (rc) return rc;
    if (!camera_ok(cam)) return fail(RTG_INVALID_PARAM, "bad camera (size, or Morton order needs multiples of 8)");
    if (!d_hits || !d_secondary_rays) return fail(RTG_INVALID_PARAM, "NULL arrays");
    cudaStream_t st = pick(s, stream);
    const int64_t n = (int64_t)cam->width * cam->height;
    if (s->hp.ncells == 0) {
        CUDA_TRY(cudaMemsetAsync(d_hits, 0xff, sizeof(rtg_hit) * n, st));
        CUDA_TRY(cudaMemsetAsync(d_secondary_rays, 0xff, 32 * n, st));
        return RTG_OK;
    }
    launch_trace_camera(view(s), camera_args(cam), reinterpret_cast<int4*>(d_hits), nullptr,
                        reinterpret_cast<float4*>(d_secondary_rays),
                        (flags & RTG_TRACE_COUNTERS) ? s->d_ctr : nullptr, next_counter(s), s->tune, s->num_sms,
                        st, 1, (unsigned long long)seed);
    CUDA_TRY(cudaGetLastError());
    return RTG_OK;
}

// GRIDRT_FUSED_FRAME = 1: rtg_trace_frame_device traces each camera ray's
// shadow ray in the same lane and launch (MODE_FRAME); 0: a camera launch,
// then an any-hit launch over the shadow-ray slots.  Same results.
#ifndef GRIDRT_FUSED_FRAME
#define GRIDRT_FUSED_FRAME 1
#endif

rtg_status rtg_trace_frame_device(rtg_scene s, const rtg_camera* cam, const float* light_pos, rtg_hit* d_hits,
                                  uint8_t* d_occ, float* d_shadow_rays, void* stream) {
    if (!light_pos || !d_occ || !d_hits) return fail(RTG_INVALID_PARAM, "NULL arguments");
    rtg_status rc = check_traceable(s, 0);
    if (rc) return rc;
    if (!camera_ok(cam)) return fail(RTG_INVALID_PARAM, "bad camera (size, or Morton order needs multiples of 8)");
    const int64_t n = (int64_t)cam->width * cam->height;
    if (!d_shadow_rays) {   // the shadow rays need a home between the two passes
        rc = ensure_io(s, 32 * n + 64);
        if (rc) return rc;
        d_shadow_rays = reinterpret_cast<float*>(s->d_io);
    }
    cudaStream_t st = pick(s, stream);
#if GRIDRT_FUSED_FRAME
    if (s->hp.ncells != 0) {
        // one launch (with its deferred passes): each lane traces its camera
        // ray, then that hit's shadow ray
        launch_trace_frame(view(s), camera_args(cam), reinterpret_cast<int4*>(d_hits), light_pos,
                           reinterpret_cast<float4*>(d_shadow_rays), d_occ, nullptr, next_counter(s), s->tune,
                           s->num_sms, st);
        CUDA_TRY(cudaGetLastError());
        return RTG_OK;
    }
#endif
    rc = rtg_trace_camera_device(s, cam, d_hits, light_pos, d_shadow_rays, 0, stream);
    if (rc) return rc;
    if (s->hp.ncells == 0) {
        CUDA_TRY(cudaMemsetAsync(d_occ, 2, n, st));
        return RTG_OK;
    }
    launch_trace_any(view(s), reinterpret_cast<const float4*>(d_shadow_rays), n, d_occ, nullptr, next_counter(s),
                     s->tune, s->num_sms, st);
    CUDA_TRY(cudaGetLastError());
    return RTG_OK;
}

rtg_status rtg_trace_frame(rtg_scene s, const rtg_camera* cam, const float* light_pos, rtg_hit* hits,
                           uint8_t* occluded, void* stream) {
    rtg_status rc = check_traceable(s, 0);
    if (rc) return rc;
    if (!camera_ok(cam)) return fail(RTG_INVALID_PARAM, "bad camera");
    if (!light_pos || !hits || !occluded) return fail(RTG_INVALID_PARAM, "NULL arguments");
    const int64_t n = (int64_t)cam->width * cam->height;
    rc = ensure_io(s, n * (16 + 32 + 1) + 64);
    if (rc) return rc;
    float* d_sr = reinterpret_cast<float*>(s->d_io);
    rtg_hit* d_hits = reinterpret_cast<rtg_hit*>(s->d_io + n * 32);
    uint8_t* d_occ = s->d_io + n * 48;
    cudaStream_t st = pick(s, stream);
    rc = rtg_trace_frame_device(s, cam, light_pos, d_hits, d_occ, d_sr, st);
    if (rc) return rc;
    CUDA_TRY(cudaMemcpyAsync(hits, d_hits, n * 16, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(occluded, d_occ, n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return RTG_OK;
}

rtg_status rtg_trace_frame_async(rtg_scene s, const rtg_camera* cam, const float* light_pos, rtg_hit* hits,
                                 uint8_t* occluded, void* stream, uint64_t* ticket) {
    rtg_status rc = check_traceable(s, 0);
    if (rc) return rc;
    if (!camera_ok(cam)) return fail(RTG_INVALID_PARAM, "bad camera");
    if (!light_pos || !hits || !occluded || !ticket) return fail(RTG_INVALID_PARAM, "NULL arguments");
    if (!s->copy_stream) {
        CUDA_TRY(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
        for (int i = 0; i < 2; ++i) {
            CUDA_TRY(cudaEventCreateWithFlags(&s->frame_traced[i], cudaEventDisableTiming));
            CUDA_TRY(cudaEventCreateWithFlags(&s->frame_copied[i], cudaEventDisableTiming));
        }
    }
    const int64_t n = (int64_t)cam->width * cam->height;
    const int64_t sr_bytes = (32 * n + 255) & ~(int64_t)255;
    const int64_t hit_bytes = (16 * n + 255) & ~(int64_t)255;
    const int64_t slot_bytes = hit_bytes + ((n + 255) & ~(int64_t)255);
    cudaStream_t st = pick(s, stream);
    if (sr_bytes + 2 * slot_bytes > s->fring_cap) {
        // a larger frame: no earlier frame of this scene may still use the ring
        CUDA_TRY(cudaStreamSynchronize(st));
        CUDA_TRY(cudaStreamSynchronize(s->copy_stream));
        CUDA_TRY(grow(s->d_fring, s->fring_cap, sr_bytes + 2 * slot_bytes));
    }
    const int slot = (int)(s->frame_seq & 1);
    float* d_sr = reinterpret_cast<float*>(s->d_fring);
    rtg_hit* d_hits = reinterpret_cast<rtg_hit*>(s->d_fring + sr_bytes + slot * slot_bytes);
    uint8_t* d_occ = s->d_fring + sr_bytes + slot * slot_bytes + hit_bytes;
    // the slot's previous frame must be copied out before this one overwrites it
    if (s->frame_seq >= 2) CUDA_TRY(cudaStreamWaitEvent(st, s->frame_copied[slot], 0));
    rc = rtg_trace_frame_device(s, cam, light_pos, d_hits, d_occ, d_sr, st);
    if (rc) return rc;
    CUDA_TRY(cudaEventRecord(s->frame_traced[slot], st));
    CUDA_TRY(cudaStreamWaitEvent(s->copy_stream, s->frame_traced[slot], 0));
    CUDA_TRY(cudaMemcpyAsync(hits, d_hits, n * 16, cudaMemcpyDeviceToHost, s->copy_stream));
    CUDA_TRY(cudaMemcpyAsync(occluded, d_occ, n, cudaMemcpyDeviceToHost, s->copy_stream));
    CUDA_TRY(cudaEventRecord(s->frame_copied[slot], s->copy_stream));
    *ticket = s->frame_seq++;
    return RTG_OK;
}

rtg_status rtg_trace_frame_wait(rtg_scene s, uint64_t ticket) {
    if (!s) return fail(RTG_INVALID_PARAM, "scene is NULL");
    if (ticket >= s->frame_seq) return fail(RTG_INVALID_PARAM, "no frame with this ticket was enqueued");
    rtg_status rc = set_device(s);
    if (rc) return rc;
    // copies finish in order on the copy stream; the slot's event marks this
    // frame's copy or a later one
    CUDA_TRY(cudaEventSynchronize(s->frame_copied[ticket & 1]));
    return RTG_OK;
}

uint64_t rtg_kernel_launch_count(void) { return (uint64_t)launches_so_far(); }

}  // extern "C"

struct rtg_batch_s {
    int device = 0;
    int num_sms = 0;
    std::vector<rtg_scene> scenes;
    std::vector<int32_t> k;
    std::vector<BuildArgs> h_build;       // host copies, to detect changed buffers
    std::vector<BatchScene> h_scenes;
    BuildArgs* d_build = nullptr;
    BatchScene* d_scenes = nullptr;
    BatchTask* d_tasks = nullptr;
    int ntasks = 0;
    long long total = 0;                   // flattened, 32-aligned ray space
    long long rays = 0;
    unsigned long long* d_counter = nullptr;   // ray claims, deferred rays, deferred claims
    int2* d_defer = nullptr;                   // deferred-ray queue (kDeferCap entries)
    TraceTuning tune;
    int* d_first = nullptr;                // kBuildKinds prefix tables of ntasks + 1 ints
    BatchGrid grid{};
    int bitmap_words = 0;
};

namespace {
// Scene buffers can be reallocated by a later synchronous build; the device
// scene table must then be refreshed before any trace reads it.
rtg_status batch_upload_views(rtg_batch b, cudaStream_t st, bool force) {
    bool changed = force;
    for (size_t i = 0; i < b->scenes.size(); ++i) {
        BatchScene v;
        v.view = view(b->scenes[i]);
        if (std::memcmp(&v, &b->h_scenes[i], sizeof(BatchScene)) != 0) {
            b->h_scenes[i] = v;
            changed = true;
        }
    }
    if (!changed) return RTG_OK;
    CUDA_TRY(cudaMemcpyAsync(b->d_scenes, b->h_scenes.data(), sizeof(BatchScene) * b->h_scenes.size(),
                             cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return RTG_OK;
}

rtg_status batch_upload_build(rtg_batch b, cudaStream_t st, bool force) {
    bool changed = force;
    for (size_t i = 0; i < b->scenes.size(); ++i) {
        BuildArgs a = make_args(b->scenes[i], b->k[i], false);
        if (std::memcmp(&a, &b->h_build[i], sizeof(BuildArgs)) != 0) {
            b->h_build[i] = a;
            changed = true;
        }
    }
    if (!changed) return RTG_OK;
    // flat batch grids: per kernel kind, the tasks' single-scene block counts back to back
    const int nt = (int)b->h_build.size();
    std::vector<int> first((size_t)kBuildKinds * (nt + 1));
    std::vector<int> blocks((size_t)nt * kBuildKinds);
    for (int t = 0; t < nt; ++t) build_blocks(b->h_build[t], b->num_sms, &blocks[(size_t)t * kBuildKinds]);
    for (int k = 0; k < kBuildKinds; ++k) first[(size_t)k * (nt + 1)] = 0;
    for (int t = 0; t < nt; ++t)
        for (int k = 0; k < kBuildKinds; ++k)
            first[(size_t)k * (nt + 1) + t + 1] = first[(size_t)k * (nt + 1) + t] + blocks[(size_t)t * kBuildKinds + k];
    for (int k = 0; k < kBuildKinds; ++k) {
        b->grid.total[k] = first[(size_t)k * (nt + 1) + nt];
        b->grid.first[k] = b->d_first + (size_t)k * (nt + 1);
    }
    b->bitmap_words = b->h_build[0].bitmap_words;
    CUDA_TRY(cudaMemcpyAsync(b->d_first, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(b->d_build, b->h_build.data(), sizeof(BuildArgs) * b->h_build.size(),
                             cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));   // the host copy may change before the next upload
    return RTG_OK;
}
}  // namespace

extern "C" {

rtg_status rtg_batch_create(const rtg_scene* scenes, int32_t nscenes, const int32_t* k, const rtg_trace_task* tasks,
                            int32_t ntasks, rtg_batch* out) {
    if (!out) return fail(RTG_INVALID_PARAM, "out is NULL");
    *out = nullptr;
    if (!scenes || nscenes <= 0 || nscenes > kMaxBatchScenes || !k || ntasks < 0 || (ntasks && !tasks))
        return fail(RTG_INVALID_PARAM, "bad batch arguments (1..64 scenes)");
    const int dev = scenes[0] ? scenes[0]->device : -1;
    for (int i = 0; i < nscenes; ++i) {
        if (!scenes[i] || scenes[i]->device != dev) return fail(RTG_INVALID_PARAM, "scenes must share one device");
        if (scenes[i]->ntris == 0 || scenes[i]->nverts == 0) return fail(RTG_INVALID_PARAM, "empty scene in batch");
        if (k[i] <= 0) return fail(RTG_INVALID_PARAM, "k must be positive");
    }
    for (int t = 0; t < ntasks; ++t) {
        const rtg_trace_task& T = tasks[t];
        if (T.scene < 0 || T.scene >= nscenes || T.n < 0 || (T.n && (!T.d_rays || !T.d_out)) ||
            (T.mode != RTG_MODE_NEAREST && T.mode != RTG_MODE_ANY))
            return fail(RTG_INVALID_PARAM, "bad trace task");
    }
    CUDA_TRY(cudaSetDevice(dev));
    for (int i = 0; i < nscenes; ++i) {   // size every scene's buffers for its grid
        rtg_status rc = rtg_scene_build(scenes[i], k[i], nullptr);
        if (rc) return rc;
    }
    rtg_batch b = new rtg_batch_s();
    b->device = dev;
    b->num_sms = scenes[0]->num_sms;
    b->scenes.assign(scenes, scenes + nscenes);
    b->k.assign(k, k + nscenes);
    b->h_build.resize(nscenes);
    b->h_scenes.resize(nscenes);
    std::vector<BatchTask> ht;
    long long first = 0;
    for (int t = 0; t < ntasks; ++t) {
        if (tasks[t].n == 0) continue;
        BatchTask T;
        T.first = first;
        T.n = tasks[t].n;
        T.rays = reinterpret_cast<const float4*>(tasks[t].d_rays);
        T.out = tasks[t].d_out;
        T.scene = tasks[t].scene;
        T.mode = tasks[t].mode;
        ht.push_back(T);
        first += (T.n + 31) / 32 * 32;
        b->rays += T.n;
    }
    b->ntasks = (int)ht.size();
    b->total = first;
    rtg_status rc = RTG_OK;
    if (cudaMalloc(&b->d_build, sizeof(BuildArgs) * nscenes) != cudaSuccess ||
        cudaMalloc(&b->d_scenes, sizeof(BatchScene) * nscenes) != cudaSuccess ||
        cudaMalloc(&b->d_tasks, sizeof(BatchTask) * (ht.size() + 1)) != cudaSuccess ||
        cudaMalloc(&b->d_counter, 3 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&b->d_defer, sizeof(int2) * kDeferCap) != cudaSuccess ||
        cudaMalloc(&b->d_first, sizeof(int) * kBuildKinds * (nscenes + 1)) != cudaSuccess)
        rc = fail(RTG_NO_MEMORY, "batch tables");
    if (rc == RTG_OK && ht.size() &&
        cudaMemcpy(b->d_tasks, ht.data(), sizeof(BatchTask) * ht.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        rc = fail(RTG_DEVICE_ERROR, "batch table upload");
    if (rc == RTG_OK) rc = batch_upload_views(b, scenes[0]->stream, true);
    if (rc == RTG_OK) rc = batch_upload_build(b, scenes[0]->stream, true);
    if (rc != RTG_OK) {
        rtg_batch_destroy(b);
        return rc;
    }
    *out = b;
    return RTG_OK;
}

rtg_status rtg_batch_build_async(rtg_batch b, void* stream) {
    if (!b) return fail(RTG_INVALID_PARAM, "batch is NULL");
    CUDA_TRY(cudaSetDevice(b->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : b->scenes[0]->stream;
    for (rtg_scene sc : b->scenes) {
        rtg_status rc = ensure_cell_records(sc);
        if (rc == RTG_OK) rc = apply_staged(sc, st);
        if (rc) return rc;
        sc->crec_built = sc->tune.cell_records != 0;   // this build writes them
    }
    rtg_status rc = batch_upload_build(b, st, false);
    if (rc == RTG_OK) rc = batch_upload_views(b, st, false);
    if (rc) return rc;
    launch_build_batch(b->d_build, (int)b->scenes.size(), b->grid, b->bitmap_words, st);
    CUDA_TRY(cudaGetLastError());
    for (rtg_scene sc : b->scenes) mark_build(sc, st);
    for (rtg_scene sc : b->scenes) sc->built = true;   // device status guards the traces
    return RTG_OK;
}

rtg_status rtg_batch_trace_async(rtg_batch b, void* stream) {
    if (!b) return fail(RTG_INVALID_PARAM, "batch is NULL");
    CUDA_TRY(cudaSetDevice(b->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : b->scenes[0]->stream;
    rtg_status rc = batch_upload_views(b, st, false);
    if (rc) return rc;
    launch_trace_batch(b->d_scenes, (int)b->scenes.size(), b->d_tasks, b->ntasks, b->total,
                       TraceSlot{b->d_counter, b->d_defer, kDeferCap}, b->tune, b->num_sms, st);
    CUDA_TRY(cudaGetLastError());
    return RTG_OK;
}

rtg_status rtg_batch_check(rtg_batch b, void* stream) {
    if (!b) return fail(RTG_INVALID_PARAM, "batch is NULL");
    CUDA_TRY(cudaSetDevice(b->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : b->scenes[0]->stream;
    CUDA_TRY(cudaStreamSynchronize(st));
    rtg_status worst = RTG_OK;
    for (rtg_scene sc : b->scenes) {
        rtg_status rc = rtg_scene_build_check(sc, nullptr);
        if (rc != RTG_OK && worst == RTG_OK) worst = rc;
    }
    return worst;
}

rtg_status rtg_batch_rays(rtg_batch b, int64_t* rays) {
    if (!b || !rays) return fail(RTG_INVALID_PARAM, "NULL argument");
    *rays = b->rays;
    return RTG_OK;
}

rtg_status rtg_batch_set_tuning(rtg_batch b, int32_t key, int32_t value) {
    if (!b) return fail(RTG_INVALID_PARAM, "batch is NULL");
    if (key == RTG_TUNE_EMPTY_RUN) {
        if (value != 2 && value != 4 && value != 8 && value != 16) return fail(RTG_INVALID_PARAM, "empty run must be 2, 4, 8 or 16");
        b->tune.empty_run = value;
        return RTG_OK;
    }
    if (key == RTG_TUNE_PERSISTENT) {
        b->tune.persistent = value ? 1 : 0;
        return RTG_OK;
    }
    if (key == RTG_TUNE_HEAVY_CELL) {
        if (value < 0) return fail(RTG_INVALID_PARAM, "heavy-cell threshold must be >= 0");
        b->tune.heavy_cell = value;
        return RTG_OK;
    }
    if (key == RTG_TUNE_HEAVY_LANES) {
        if (value != 4 && value != 8 && value != 16 && value != 32)
            return fail(RTG_INVALID_PARAM, "heavy lanes must be 4, 8, 16 or 32");
        b->tune.heavy_lanes = value;
        return RTG_OK;
    }
    if (key == RTG_TUNE_REFILL) {
        if (value < 0 || value > 32) return fail(RTG_INVALID_PARAM, "refill threshold must be 0..32");
        b->tune.refill = value;
        return RTG_OK;
    }
    return fail(RTG_INVALID_PARAM, "unknown tuning key");
}

rtg_status rtg_batch_destroy(rtg_batch b) {
    if (!b) return RTG_OK;
    cudaSetDevice(b->device);
    cudaDeviceSynchronize();
    cudaFree(b->d_build);
    cudaFree(b->d_scenes);
    cudaFree(b->d_tasks);
    cudaFree(b->d_counter);
    cudaFree(b->d_defer);
    cudaFree(b->d_first);
    delete b;
    return RTG_OK;
}

rtg_status rtg_scene_set_tuning(rtg_scene s, int32_t key, int32_t value) {
    if (!s) return fail(RTG_INVALID_PARAM, "scene is NULL");
    switch (key) {
        case RTG_TUNE_EMPTY_RUN:
            if (value != 2 && value != 4 && value != 8 && value != 16) return fail(RTG_INVALID_PARAM, "empty run must be 2, 4, 8 or 16");
            s->tune.empty_run = value;
            return RTG_OK;
        case RTG_TUNE_PERSISTENT:
            s->tune.persistent = value ? 1 : 0;
            return RTG_OK;
        case RTG_TUNE_HEAVY_CELL:
            if (value < 0) return fail(RTG_INVALID_PARAM, "heavy-cell threshold must be >= 0");
            if (value > 0 && !s->d_defer) {
                CUDA_TRY(cudaSetDevice(s->device));
                if (cudaMalloc(&s->d_defer, kDeferAlloc) != cudaSuccess) {
                    s->d_defer = nullptr;
                    return fail(RTG_NO_MEMORY, "deferred-ray queues");
                }
            }
            s->tune.heavy_cell = value;
            return RTG_OK;
        case RTG_TUNE_HEAVY_LANES:
            if (value != 4 && value != 8 && value != 16 && value != 32)
                return fail(RTG_INVALID_PARAM, "heavy lanes must be 4, 8, 16 or 32");
            s->tune.heavy_lanes = value;
            return RTG_OK;
        case RTG_TUNE_CELL_RECORDS:
            // takes effect at the next build (which then also writes the records)
            s->tune.cell_records = value ? 1 : 0;
            if (!value) s->crec_built = false;
            return RTG_OK;
        case RTG_TUNE_REFILL:
            if (value < 0 || value > 32) return fail(RTG_INVALID_PARAM, "refill threshold must be 0..32");
            s->tune.refill = value;
            return RTG_OK;
        case RTG_TUNE_BLOCK:
            if (value != 64 && value != 128 && value != 256)
                return fail(RTG_INVALID_PARAM, "trace block size must be 64, 128 or 256");
            s->tune.block = value;
            return RTG_OK;
        case RTG_TUNE_LANES:
            if (value != 1 && value != 2 && value != 4)
                return fail(RTG_INVALID_PARAM, "lanes per ray must be 1, 2 or 4");
            s->tune.lanes = value;
            return RTG_OK;
        default:
            return fail(RTG_INVALID_PARAM, "unknown tuning key");
    }
}

rtg_status rtg_scene_counters(rtg_scene s, int64_t out[3], int reset) {
    if (!s || !out) return fail(RTG_INVALID_PARAM, "NULL argument");
    rtg_status rc = set_device(s);
    if (rc) return rc;
    TraceCounters c;
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    CUDA_TRY(cudaDeviceSynchronize());
    CUDA_TRY(cudaMemcpy(&c, s->d_ctr, sizeof(c), cudaMemcpyDeviceToHost));
    out[0] = (int64_t)c.rays;
    out[1] = (int64_t)c.cells;
    out[2] = (int64_t)c.tests;
    if (reset) CUDA_TRY(cudaMemset(s->d_ctr, 0, sizeof(c)));
    return RTG_OK;
}

}  // extern "C"
