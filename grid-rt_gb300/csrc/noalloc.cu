// noalloc.cu -- grid build that allocates no device memory.
//
// Some callers cannot let a library call cudaMalloc: a real-time frame loop
// where an allocation (and the device synchronisation it can imply) would
// stall the frame, or a host application that owns every byte of device
// memory through its own pool or allocator and budgets it.  For them,
// rtg_grid_build_noalloc builds the uniform grid straight into buffers the
// caller passes, and keeps all of the build's working memory (grid
// parameters, bounding-box keys, scan tile sums, sort work lists and the
// large-cell sort copy) in one file-scope device array of fixed size.
//
// Limits: at most kMaxRefs (cell, triangle) references and kMaxCells cells per
// build.  The array occupies kArenaBytes on every GPU that loads the library,
// until the process exits.
//
// Every call uses the same array: the call clears the parts that must start
// at zero (or all-ones) before its kernels run, and calls whose work overlaps
// on the GPU -- on different streams, or from different host threads at once
// -- race on the array.  Serialise them (one stream, or wait between calls).
//
// Set-up: every call looks up the array's device address with
// cudaGetSymbolAddress on the device that is current, and sets the large-cell
// sort kernel's shared-memory limit there (so a call after cudaDeviceReset
// finds the new context's address); the first call on a device also reads
// its SM count and shared-memory limit.  Make that first call before any
// stream capture begins on the device.
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/gridrt.h"
#include "common.cuh"
#include "kernels.h"

namespace gridrt {
namespace {

constexpr int64_t kMaxRefs = int64_t(1) << 19;    // 524,288 references
constexpr int64_t kMaxCells = int64_t(1) << 24;   // 16,777,216 cells (tile sums)

// Arena layout (byte offsets; every part 256-byte aligned).
constexpr size_t kOffParams = 0;
constexpr size_t kOffWork = 256;
constexpr size_t kOffTiles = 512;
constexpr size_t kTileCount = kMaxCells / kScanTile + 2;
constexpr size_t kOffQSmall = kOffTiles + ((kTileCount * 8 + 255) / 256) * 256;
constexpr size_t kQSmall = kMaxRefs / 2 + 2;
constexpr size_t kOffQMed = kOffQSmall + ((kQSmall * 4 + 255) / 256) * 256;
constexpr size_t kQMed = kMaxRefs / 33 + 2;
constexpr size_t kOffQLarge = kOffQMed + ((kQMed * 4 + 255) / 256) * 256;
constexpr size_t kQLarge = kMaxRefs / (SORT_MED_MAX + 1) + 2;
constexpr size_t kOffScratch = kOffQLarge + ((kQLarge * 4 + 255) / 256) * 256;
constexpr size_t kArenaBytes = kOffScratch + kMaxRefs * 4;

static_assert(sizeof(GridParams) <= 256, "params slot");
static_assert(sizeof(BuildWork) <= 256, "work slot");

// The build's working memory.  In host code this name is only a host-side
// stand-in for the symbol: the device address comes from
// cudaGetSymbolAddress below and is what the kernels receive.
static __device__ __align__(256) unsigned char g_noalloc_arena[kArenaBytes];

struct DeviceSetup {
    bool ready = false;
    unsigned char* arena = nullptr;
    int num_sms = 0;
    int bitmap_words = 0;
};

std::mutex g_setup_mutex;
DeviceSetup g_setup[64];

rtg_status failure(rtg_status s, const char* what, cudaError_t e = cudaSuccess) {
    std::string msg = what;
    if (e != cudaSuccess) {
        msg += ": ";
        msg += cudaGetErrorString(e);
    }
    set_last_error(msg);   // reported by rtg_last_error()
    return s;
}

rtg_status setup_device(int dev, DeviceSetup** out) {
    if (dev < 0 || dev >= 64) return failure(RTG_INVALID_PARAM, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceSetup& d = g_setup[dev];
    if (!d.ready) {
        int sms = 0, optin = 0;
        cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return failure(RTG_DEVICE_ERROR, "SM count", e);
        e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e != cudaSuccess) return failure(RTG_DEVICE_ERROR, "shared-memory limit", e);
        int words = 32768;
        while (words * 4 + 4096 > optin && words > 1024) words >>= 1;
        d.num_sms = sms;
        d.bitmap_words = words;
        d.ready = true;
    }
    // The array's address and the large-cell sort's shared-memory limit
    // belong to the device's current context: a device reset
    // (cudaDeviceReset) gives the next call a new context, in which the
    // array may sit elsewhere and the kernel's attribute is back at its
    // default.  So every call looks the address up again and re-applies the
    // attribute (both host-side calls of a few microseconds).
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_arena);
    if (e != cudaSuccess || !ptr) return failure(RTG_DEVICE_ERROR, "cudaGetSymbolAddress(arena)", e);
    e = build_setup_attributes(d.bitmap_words);
    if (e != cudaSuccess) return failure(RTG_DEVICE_ERROR, "large-cell sort attribute", e);
    d.arena = static_cast<unsigned char*>(ptr);
    *out = &d;
    return RTG_OK;
}

void fill_info(const GridParams& p, int32_t k, rtg_grid_info* info) {
    std::memset(info, 0, sizeof(*info));
    for (int a = 0; a < 3; ++a) {
        info->res[a] = p.res[a];
        info->bmin[a] = p.bmin[a];
        info->bmax[a] = p.bmax[a];
        info->cell[a] = p.cell[a];
        info->inv_cell[a] = p.inv[a];
    }
    info->ncells = p.ncells;
    info->nrefs = p.nrefs;
    info->k = k;
}

}  // namespace
}  // namespace gridrt

using namespace gridrt;

extern "C" rtg_status rtg_grid_build_noalloc(const float* d_verts, int64_t nverts, const int32_t* d_tris,
                                             int64_t ntris, int32_t k, int32_t* d_offsets, int64_t offsets_cap,
                                             int32_t* d_ids, int64_t ids_cap, float* d_tri_records,
                                             rtg_grid_info* info, void* stream) {
    if (!info) return failure(RTG_INVALID_PARAM, "info is NULL");
    std::memset(info, 0, sizeof(*info));
    if (k <= 0 || nverts < 0 || ntris < 0 || offsets_cap < 1 || ids_cap < 0)
        return failure(RTG_INVALID_PARAM, "bad sizes");
    if (!d_offsets || (ntris > 0 && (!d_verts || !d_tris || !d_tri_records || !d_ids)))
        return failure(RTG_INVALID_PARAM, "NULL array");
    if ((reinterpret_cast<uintptr_t>(d_offsets) & 15) || (reinterpret_cast<uintptr_t>(d_tri_records) & 15))
        return failure(RTG_INVALID_PARAM, "offsets and triangle records must be 16-byte aligned");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return failure(RTG_DEVICE_ERROR, "cudaGetDevice", e);
    DeviceSetup* d = nullptr;
    rtg_status rc = setup_device(dev, &d);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    info->k = k;
    if (ntris == 0 || nverts == 0) {   // empty grid, as rtg_scene_build reports it
        e = cudaMemsetAsync(d_offsets, 0, sizeof(int32_t), st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        return e == cudaSuccess ? RTG_OK : failure(RTG_DEVICE_ERROR, "clear offsets", e);
    }

    GridParams* params = reinterpret_cast<GridParams*>(d->arena + kOffParams);
    BuildWork* work = reinterpret_cast<BuildWork*>(d->arena + kOffWork);
    // Clear what must start fresh: parameters and the work block (min keys
    // start at all-ones, everything else at zero).
    e = cudaMemsetAsync(params, 0, sizeof(GridParams), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(work, 0, sizeof(BuildWork), st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(reinterpret_cast<unsigned char*>(work) + offsetof(BuildWork, keys), 0xff,
                            3 * sizeof(uint32_t), st);
    if (e != cudaSuccess) return failure(RTG_DEVICE_ERROR, "clear arena", e);

    BuildArgs a;
    a.verts = d_verts;
    a.nverts = nverts;
    a.idx = d_tris;
    a.ntris = ntris;
    a.k = k;
    a.skip_bbox = false;
    a.params = params;
    a.work = work;
    a.tris = reinterpret_cast<float4*>(d_tri_records);
    a.wald = nullptr;  // hit-value records serve only the scene's trace kernels
    a.offsets = d_offsets;
    a.occ = nullptr;   // the occupancy bitmap only serves the scene's trace kernels
    a.crec = nullptr;
    a.cell_cap = offsets_cap < kMaxCells + 1 ? offsets_cap : kMaxCells + 1;
    a.ids = d_ids;
    a.scratch = reinterpret_cast<int32_t*>(d->arena + kOffScratch);
    a.ref_cap = ids_cap < kMaxRefs ? ids_cap : kMaxRefs;
    a.tile_sums = reinterpret_cast<int64_t*>(d->arena + kOffTiles);
    a.q_small = reinterpret_cast<int32_t*>(d->arena + kOffQSmall);
    a.q_med = reinterpret_cast<int32_t*>(d->arena + kOffQMed);
    a.q_large = reinterpret_cast<int32_t*>(d->arena + kOffQLarge);
    a.q_small_cap = (int64_t)kQSmall;
    a.q_med_cap = (int64_t)kQMed;
    a.q_large_cap = (int64_t)kQLarge;
    a.bitmap_words = d->bitmap_words;
    a.num_sms = d->num_sms;

    GridParams hp;
    for (int attempt = 0; attempt < 2; ++attempt) {
        launch_build(a, st);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(&hp, params, sizeof(GridParams), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return failure(RTG_DEVICE_ERROR, "build", e);
        if (!(hp.status & ST_AMBIGUOUS) || attempt == 1) break;
        // The last ulp of powf decides a cell count: resolve on the host with
        // the C library's powf, then rerun everything after the box.
        host_resolve(hp, k, ntris, a.cell_cap);
        e = cudaMemcpyAsync(params, &hp, sizeof(GridParams), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(reinterpret_cast<unsigned char*>(work) + offsetof(BuildWork, nsort), 0,
                                sizeof(BuildWork::nsort), st);
        if (e != cudaSuccess) return failure(RTG_DEVICE_ERROR, "upload resolved parameters", e);
        if (hp.status & (ST_CELL_CAP | ST_TOO_BIG)) break;
        a.skip_bbox = true;
    }
    fill_info(hp, k, info);
    if (hp.status & ST_TOO_BIG) return failure(RTG_INVALID_PARAM, "grid exceeds the int32 index space");
    if (hp.status & ST_CELL_CAP) {
        if (hp.ncells + 1 > kMaxCells + 1) return failure(RTG_INVALID_PARAM, "more cells than the no-allocation limit");
        return failure(RTG_NO_MEMORY, "offsets buffer too small (info->ncells + 1 entries needed)");
    }
    if (hp.status & (ST_REF_CAP | ST_SORT_CAP)) {
        if (hp.nrefs > kMaxRefs) return failure(RTG_INVALID_PARAM, "more references than the no-allocation limit");
        return failure(RTG_NO_MEMORY, "ids buffer too small (info->nrefs entries needed)");
    }
    if (hp.status & ST_BAD_RANGE) return failure(RTG_INVALID_GEOMETRY, "non-finite vertex or triangle outside the grid");
    info->built = 1;
    return RTG_OK;
}
