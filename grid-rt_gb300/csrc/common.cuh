// common.cuh -- shared device types and exact-rounding helpers.
//
// Parity-critical arithmetic (grid parameters, cell ranges, ray setup, box
// clip, 3D-DDA) must round exactly like the reference's float code, which
// evaluates every + - * / once in IEEE single precision
// (src/rtplugins/UniformGridAccStruct.cpp:92-103,113-196,
//  src/rtcore/AabbIntersection.cpp:37-63, include/rt/Ray.h:26-37).
// The helpers below use the _rn intrinsics so nvcc can never contract them
// into FMAs.  The Moller-Trumbore test is not bit-compared and may use FMA.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gridrt {

// Grid parameters as UniformGridAccStruct holds them
// (include/rtp/UniformGridAccStruct.h:49-56 + IAccStruct::_bbox).
struct GridParams {
    float bmin[3];
    float bmax[3];
    float cell[3];
    float inv[3];
    int32_t res[3];
    int32_t k;
    int64_t ncells;
    int64_t nrefs;
    int64_t ntris;
    uint32_t status;
    uint32_t max_list;    // longest cell list of the build (set by the scan)
};

// status bits written by the build kernels
enum : uint32_t {
    ST_CELL_CAP = 1u,     // ncells + 1 exceeds the offsets capacity
    ST_REF_CAP = 2u,      // nrefs exceeds the ids capacity
    ST_BAD_RANGE = 4u,    // a triangle's cell range fell outside the grid (non-finite input)
    ST_AMBIGUOUS = 8u,    // resolution depends on the last ulp of powf: host recomputes
    ST_TOO_BIG = 16u,     // ncells or nrefs beyond int32 (the reference's index type)
    ST_SORT_CAP = 32u,    // segmented-sort work lists overflowed
};

// Programmatic dependent launch (GRIDRT_PDL = 1): build and trace kernels are
// launched with programmatic stream serialisation, so a kernel's blocks may
// be scheduled while its predecessor drains; every such kernel first waits
// (griddepcontrol.wait) until the predecessor has completed and its memory
// is visible, then allows its own successor to start launching.  Without the
// launch attribute both instructions return at once.  On by default: frames
// launched call by call run 5% faster (0.459 -> 0.437 ms, deforming sphere
// k = 2); graph-replayed frames are unchanged.
#ifndef GRIDRT_PDL
#define GRIDRT_PDL 1
#endif
__device__ __forceinline__ void pdl_begin() {
#if GRIDRT_PDL
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

// Per-cell sort size classes: one thread's registers up to 8 entries, warp
// registers up to 32, one warp's registers up to 256, a block above (bitonic
// up to 4096, bitmap beyond).
static constexpr int SORT_TINY_MAX = 8;
static constexpr int SORT_SMALL_MAX = 32;
static constexpr int SORT_MED_MAX = 256;
static constexpr int SORT_BLOCK_MAX = 4096;

// Work state shared by the build kernels of one scene (device memory).
struct BuildWork {
    uint32_t keys[6];        // ordered-int min xyz, max xyz
    uint32_t ticket;         // last-block ticket of the bbox kernel
    uint32_t nsort[4];       // cells queued: 2..8 entries (front of the small queue), 33..256, above 256,
                             // 9..32 (back of the small queue)
    uint32_t sticky;         // OR of every build's status since the host last cleared it
    uint32_t pad[4];
};

static constexpr float kHitEpsilon = 1e-4f;   // src/rtcore/RayTriIntersection.cpp:6
static constexpr float kRayEpsilon = 2e-4f;   // src/rtcore/Context.cpp:505
static constexpr float kFltMax = 3.402823466e+38f;

// Sets status bits on the current build and on the sticky word.
__device__ __forceinline__ void raise_status(GridParams* p, BuildWork* w, uint32_t bits) {
    atomicOr(&p->status, bits);
    if (w) atomicOr(&w->sticky, bits);
}

static __host__ __device__ __forceinline__ bool build_failed(uint32_t s) {
    return (s & (ST_CELL_CAP | ST_AMBIGUOUS | ST_TOO_BIG | ST_REF_CAP | ST_SORT_CAP | ST_BAD_RANGE)) != 0;
}

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float frcp(float a) { return __frcp_rn(a); }
// vr::min / vr::max / vr::abs semantics (a < b ? a : b etc.)
__device__ __forceinline__ float vmin(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float vmax(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float vabs(float x) { return x < 0.0f ? -x : x; }
__device__ __forceinline__ int32_t vclamp(int32_t v, int32_t lo, int32_t hi) { return v < lo ? lo : (v > hi ? hi : v); }

// UniformGridAccStruct::worldToVoxel (float -> int32 truncation toward zero)
__device__ __forceinline__ int32_t world_to_voxel(float v, float bmin, float inv) {
    return __float2int_rz(fmul(fsub(v, bmin), inv));
}
// UniformGridAccStruct::voxelToWorld
__device__ __forceinline__ float voxel_to_world(int32_t vox, float cell, float bmin) {
    return fadd(fmul(__int2float_rn(vox), cell), bmin);
}

// Occupancy bitmap: one bit per cell, 32 cells per word grouped in 4x4x2
// bricks so a DDA walk keeps using one word for several steps in any
// direction.  Word count never exceeds the cell count.
__host__ __device__ __forceinline__ int64_t occ_words(int32_t nx, int32_t ny, int32_t nz) {
    return (int64_t)((nx + 3) >> 2) * ((ny + 3) >> 2) * ((nz + 1) >> 1);
}
__device__ __forceinline__ uint32_t occ_bit(int32_t x, int32_t y, int32_t z) {
    return 1u << ((x & 3) | ((y & 3) << 2) | ((z & 1) << 4));
}

// Monotone float <-> uint32 key for atomicMin / atomicMax.
__device__ __forceinline__ uint32_t f2key(float f) {
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key2f(uint32_t k) {
    uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(b);
}

}  // namespace gridrt
