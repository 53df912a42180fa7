// trace_device.cuh -- one-ray-per-thread 3D-DDA traversal (device code of the
// tracer and its single-scene launch helpers, shared by its translation units).
//
// Replaces rtp::UniformGridAccStruct::traceNearestGeometry / traverse3ddda
// (src/rtplugins/UniformGridAccStruct.cpp:30-42, 113-196, 362-378) and the
// reference's GPU tracers (src/rtcuda/RayTracing_kernel.cu:140-275,
// shaders/traversalIntersection_FRAG.glsl:161-263, shaders/shadow_FRAG.glsl:147-245).
//
// The DDA follows the CPU reference exactly -- integer cells, strict-< axis
// choice, exit test x != outX && y != outY && z != outZ, per-cell acceptance
// window [tnear - 1e-4, cellExit + 1e-4] (src/rtcore/RayTriIntersection.cpp:20),
// first cell with a hit ends the walk -- so the visited cells and the tested
// triangles are the reference's.  Each test is Moller-Trumbore, which rejects
// the triangles a ray clearly misses; the candidates it leaves are decided by
// the reference's own projection test on the triangle's TriAccel record, so
// the decisions and the reported t / u / v are the reference's.
//
// Execution: persistent warps.  A warp claims 32 consecutive rays with one
// global atomicAdd, traces them to the end (one ray per lane; consecutive
// camera rays in Morton order stay coherent) and claims the next 32, so no
// warp idles while a block-mate finishes (or, with lane refill, hands new
// rays to its idle lanes as it goes).  Per loop iteration a lane walks up to
// ER empty cells (a tuning parameter), decided from a 4x4x2-brick occupancy
// bitmap whose current word stays in a register, and tests at most one
// non-empty cell, so lanes that reach triangles test them together.  A frame
// (MODE_FRAME) traces each camera ray's shadow ray in the same lane right
// after it.  Rays that meet a long list finish in a group-of-lanes pass,
// those that then meet a dense cluster's list in a block-per-ray pass.
#pragma once

#include "common.cuh"
#include "kernels.h"

namespace gridrt {

static constexpr unsigned FULL = 0xffffffffu;
static constexpr int32_t kDeferred = -3;    // Lane::id of a ray handed to the warp-per-ray pass
static constexpr int32_t kNoHeavy = 0x7fffffff;
static constexpr int kWideEmptyRun = 8;     // empty cells a deferred ray's group walks per turn
// A ray is also deferred once its tests would pass kHeavyWorkMult x the
// heavy-cell threshold in total (0: only long lists defer).
#ifndef GRIDRT_HEAVY_WORK_MULT
#define GRIDRT_HEAVY_WORK_MULT 8
#endif
static constexpr int32_t kHeavyWorkMult = GRIDRT_HEAVY_WORK_MULT;


// MODE_FRAME: a camera ray, then in the same lane the shadow ray of its hit
// (any-hit); Lane::tmax is -inf in the camera phase and the shadow ray's
// tmax after.
enum Mode : int { MODE_NEAREST = 0, MODE_ANY = 1, MODE_CAMERA = 2, MODE_FRAME = 3 };

struct SParams {
    float bmin[3], bmax[3], cell[3], inv[3];
    int32_t res[3];
    int32_t bx, bxby;
    int32_t failed;
};

__device__ __forceinline__ void fill_sparams(const GridParams* __restrict__ gp, SParams& P) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        P.bmin[d] = gp->bmin[d];
        P.bmax[d] = gp->bmax[d];
        P.cell[d] = gp->cell[d];
        P.inv[d] = gp->inv[d];
        P.res[d] = gp->res[d];
    }
    P.bx = (P.res[0] + 3) >> 2;
    P.bxby = P.bx * ((P.res[1] + 3) >> 2);
    P.failed = build_failed(gp->status) ? 1 : 0;
}

__device__ __forceinline__ void load_sparams(const GridParams* __restrict__ gp, SParams& P) {
    if (threadIdx.x == 0) fill_sparams(gp, P);
    __syncthreads();
}

// Live state of one ray (registers).
struct Lane {
    float ox, oy, oz, dx, dy, dz;
    float ix, iy, iz;
    float tmax, lo;
    float tMx, tMy, tMz, tDx, tDy, tDz;
    int32_t x, y, z;
    int32_t budget;
    int32_t work;        // triangle tests made so far by this ray
    float best;
    int32_t id;
    int32_t cw;          // cached occupancy word index
    uint32_t cword;      // its value
    int32_t ray;         // ray index within the launch or task, -1 = none
};

// Ray::update + AabbIntersection::clipRay + traverse3ddda set-up
// (include/rt/Ray.h:26-37, src/rtcore/AabbIntersection.cpp:37-63,
//  src/rtplugins/UniformGridAccStruct.cpp:122-149).  False if the ray misses
// the grid box.
__device__ __forceinline__ bool setup_ray(const SParams& P, Lane& L, float tnear, float tfar) {
    L.ix = frcp(L.dx);
    L.iy = frcp(L.dy);
    L.iz = frcp(L.dz);
    L.tmax = tfar;
    float rn = tnear, rf = tfar;
    {
        float tn = fmul(fsub(P.bmin[0], L.ox), L.ix), tf = fmul(fsub(P.bmax[0], L.ox), L.ix);
        rn = vmax(rn, vmin(tn, tf));
        rf = vmin(rf, vmax(tn, tf));
        tn = fmul(fsub(P.bmin[1], L.oy), L.iy);
        tf = fmul(fsub(P.bmax[1], L.oy), L.iy);
        rn = vmax(rn, vmin(tn, tf));
        rf = vmin(rf, vmax(tn, tf));
        tn = fmul(fsub(P.bmin[2], L.oz), L.iz);
        tf = fmul(fsub(P.bmax[2], L.oz), L.iz);
        rn = vmax(rn, vmin(tn, tf));
        rf = vmin(rf, vmax(tn, tf));
    }
    if (rn > rf) return false;
    L.lo = fsub(rn, kHitEpsilon);
    const int32_t sx = __float_as_uint(L.dx) >> 31, sy = __float_as_uint(L.dy) >> 31, sz = __float_as_uint(L.dz) >> 31;
    L.x = vclamp(world_to_voxel(fadd(L.ox, fmul(L.dx, rn)), P.bmin[0], P.inv[0]), 0, P.res[0] - 1);
    L.y = vclamp(world_to_voxel(fadd(L.oy, fmul(L.dy, rn)), P.bmin[1], P.inv[1]), 0, P.res[1] - 1);
    L.z = vclamp(world_to_voxel(fadd(L.oz, fmul(L.dz, rn)), P.bmin[2], P.inv[2]), 0, P.res[2] - 1);
    L.tDx = vabs(fmul(P.cell[0], L.ix));
    L.tDy = vabs(fmul(P.cell[1], L.iy));
    L.tDz = vabs(fmul(P.cell[2], L.iz));
    L.tMx = fmul(fsub(voxel_to_world(L.x + (sx ^ 1), P.cell[0], P.bmin[0]), L.ox), L.ix);
    L.tMy = fmul(fsub(voxel_to_world(L.y + (sy ^ 1), P.cell[1], P.bmin[1]), L.oy), L.iy);
    L.tMz = fmul(fsub(voxel_to_world(L.z + (sz ^ 1), P.cell[2], P.bmin[2]), L.oz), L.iz);
    // A walk visits at most nx+ny+nz-2 cells; the bound only guards against a
    // zero direction component (outside the reference's domain) looping.
    L.budget = P.res[0] + P.res[1] + P.res[2] + 3;
    L.work = 0;
    L.best = kFltMax;
    L.id = -1;
    L.cw = -1;
    return true;
}

#ifndef GRIDRT_EXIT_ALL
#define GRIDRT_EXIT_ALL 0
#endif

// One DDA step (src/rtplugins/UniformGridAccStruct.cpp:179-195): the strict-<
// axis choice and a step of vr::sign(direction).  The reference then exits
// when x == outX (or y, z), with out = -1 for a negative direction sign bit and
// n otherwise (:137-139, :195).  A walk starts inside the grid and moves each
// coordinate only toward its out value, so it reaches out exactly when the
// coordinate leaves [0, n): the test below is the same predicate.  True when
// the walk has left the grid.
__device__ __forceinline__ bool dda_step(const SParams& P, Lane& L) {
    // the other two coordinates did not move and were inside: only the moved
    // one can have left the grid
    bool out;
    if (L.tMx < L.tMy && L.tMx < L.tMz) {
        L.x += L.dx < 0.0f ? -1 : (L.dx > 0.0f ? 1 : 0);
        L.tMx = fadd(L.tMx, L.tDx);
        out = (unsigned)L.x >= (unsigned)P.res[0];
    } else if (L.tMy < L.tMz) {
        L.y += L.dy < 0.0f ? -1 : (L.dy > 0.0f ? 1 : 0);
        L.tMy = fadd(L.tMy, L.tDy);
        out = (unsigned)L.y >= (unsigned)P.res[1];
    } else {
        L.z += L.dz < 0.0f ? -1 : (L.dz > 0.0f ? 1 : 0);
        L.tMz = fadd(L.tMz, L.tDz);
        out = (unsigned)L.z >= (unsigned)P.res[2];
    }
#if GRIDRT_EXIT_ALL
    out = (unsigned)L.x >= (unsigned)P.res[0] || (unsigned)L.y >= (unsigned)P.res[1] ||
          (unsigned)L.z >= (unsigned)P.res[2];
#endif
    return out || --L.budget <= 0;
}

// Triangle test.  Moller-Trumbore on the triangle's {v0, e1, e2} record
// rejects every triangle the ray clearly misses; a triangle that passes it
// within the slacks below -- its barycentrics within kMtBarySlack of the
// triangle, its t within kMtTRelSlack (relative) + 1e-4 of the acceptance
// window and of the best hit so far -- is decided by the reference's own test
// (RayTriIntersection::hitWald, src/rtcore/RayTriIntersection.cpp:12-48) on
// its TriAccel record, in the reference's operation order and rounding.  So
// every accept / reject decision, and the best distance carried from test to
// test, are the reference's: the two float tests round differently near an
// edge or a window bound, but only Wald's decides.  Moller-Trumbore's own
// error stays far inside the slacks (its barycentric error is below 1e-5 for
// the workloads' triangles; a triangle would need a far larger
// distance-to-size ratio for the filter to drop a hit that Wald accepts).
// Returns true when ANY mode found a hit before tmax.
// GRIDRT_MT_EARLY_OUT = 1 lets a lane leave once u (then v) fails.
// GRIDRT_MT_FAST_RCP = 1 takes the filter's 1/det from the hardware's
// approximate reciprocal (rcp.approx), well inside the slacks.
// GRIDRT_DECIDE_WALD = 0 restores plain Moller-Trumbore decisions (ids then
// differ from the reference's at near-ties; the reported values stay Wald's).
#ifndef GRIDRT_MT_EARLY_OUT
#define GRIDRT_MT_EARLY_OUT 1
#endif
#ifndef GRIDRT_MT_FAST_RCP
#define GRIDRT_MT_FAST_RCP 1
#endif
#ifndef GRIDRT_DECIDE_WALD
#define GRIDRT_DECIDE_WALD 1
#endif
static constexpr float kMtBarySlack = GRIDRT_DECIDE_WALD ? 1e-2f : 0.0f;
static constexpr float kMtTRelSlack = 1e-3f;

__device__ __forceinline__ float pick3(float x, float y, float z, uint32_t d) {
    return d == 0 ? x : (d == 1 ? y : z);
}

// hitWald's decision (and f) for triangle `tid` against the lane's ray and
// best distance, window [L.lo, hi].
template <int MODE>
__device__ __forceinline__ bool wald_decide(Lane& L, int32_t tid, float hi, const float4* __restrict__ wald) {
    const float4 a0 = __ldg(wald + 3 * (int64_t)tid);
    const uint32_t k = __float_as_uint(a0.x);
    const uint32_t ku = k == 2 ? 0 : k + 1, kv = k == 0 ? 2 : k - 1;
    const float dk = pick3(L.dx, L.dy, L.dz, k), du = pick3(L.dx, L.dy, L.dz, ku), dv = pick3(L.dx, L.dy, L.dz, kv);
    const float ok = pick3(L.ox, L.oy, L.oz, k), ou = pick3(L.ox, L.oy, L.oz, ku), ov = pick3(L.ox, L.oy, L.oz, kv);
    const float nd = frcp(fadd(fadd(dk, fmul(a0.y, du)), fmul(a0.z, dv)));
    const float f = fmul(nd, fsub(fsub(fsub(a0.w, ok), fmul(a0.y, ou)), fmul(a0.z, ov)));
    if ((f >= L.best) || (f < L.lo) || (f > hi)) return false;
    const float4 a1 = __ldg(wald + 3 * (int64_t)tid + 1);
    const float hu = fadd(ou, fmul(f, du));
    const float hv = fadd(ov, fmul(f, dv));
    const float lambda = fadd(fadd(fmul(hu, a1.x), fmul(hv, a1.y)), a1.z);
    if (lambda < 0.0f) return false;
    const float4 a2 = __ldg(wald + 3 * (int64_t)tid + 2);
    const float mue = fadd(fadd(fmul(hu, a2.x), fmul(hv, a2.y)), a2.z);
    if (mue < 0.0f) return false;
    if (fsub(fsub(1.0f, lambda), mue) < 0.0f) return false;
    L.best = f;
    L.id = tid;
    return (MODE == MODE_ANY || MODE == MODE_FRAME) && f < L.tmax;
}

template <int MODE>
__device__ __forceinline__ bool test_tri(Lane& L, int32_t tid, const float4& A, const float4& B, const float4& C,
                                         float hi, const float4* __restrict__ wald) {
    const float tvx = L.ox - A.x, tvy = L.oy - A.y, tvz = L.oz - A.z;
    const float px = L.dy * C.z - L.dz * C.y;
    const float py = L.dz * C.x - L.dx * C.z;
    const float pz = L.dx * C.y - L.dy * C.x;
    const float det = B.x * px + B.y * py + B.z * pz;
#if GRIDRT_MT_FAST_RCP
    float idet;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(idet) : "f"(det));
#else
    const float idet = frcp(det);
#endif
    const float u = (tvx * px + tvy * py + tvz * pz) * idet;
#if GRIDRT_MT_EARLY_OUT
    // the same predicate, decided in stages: a lane leaves after u
    if (!(u >= -kMtBarySlack)) return false;
#endif
    const float qx = tvy * B.z - tvz * B.y;
    const float qy = tvz * B.x - tvx * B.z;
    const float qz = tvx * B.y - tvy * B.x;
    const float v = (L.dx * qx + L.dy * qy + L.dz * qz) * idet;
#if GRIDRT_MT_EARLY_OUT
    if (!(v >= -kMtBarySlack && (1.0f - u) - v >= -kMtBarySlack)) return false;
#endif
    const float t = (C.x * qx + C.y * qy + C.z * qz) * idet;
#if GRIDRT_DECIDE_WALD
    const float ts = fabsf(t) * kMtTRelSlack + kHitEpsilon;
    if (!((t < L.best + ts) && (t >= L.lo - ts) && (t <= hi + ts) && (u >= -kMtBarySlack) &&
          (v >= -kMtBarySlack) && ((1.0f - u) - v >= -kMtBarySlack)))
        return false;
    return wald_decide<MODE>(L, tid, hi, wald);
#else
    const bool acc = (t < L.best) && (t >= L.lo) && (t <= hi) && (u >= 0.0f) && (v >= 0.0f) &&
                     ((1.0f - u) - v >= 0.0f);
    if (acc) {
        L.best = t;
        L.id = tid;
        if ((MODE == MODE_ANY || MODE == MODE_FRAME) && t < L.tmax) return true;
    }
    return false;
#endif
}

// hitWald's f alone (the exact distance of a hit that test_tri_fast accepted
// without the reference's test, when a later decision compares against it).
__device__ __forceinline__ float wald_f_of(const Lane& L, int32_t tid, const float4* __restrict__ wald) {
    const float4 a0 = __ldg(wald + 3 * (int64_t)tid);
    const uint32_t k = __float_as_uint(a0.x);
    const uint32_t ku = k == 2 ? 0 : k + 1, kv = k == 0 ? 2 : k - 1;
    const float dk = pick3(L.dx, L.dy, L.dz, k), du = pick3(L.dx, L.dy, L.dz, ku), dv = pick3(L.dx, L.dy, L.dz, kv);
    const float ok = pick3(L.ox, L.oy, L.oz, k), ou = pick3(L.ox, L.oy, L.oz, ku), ov = pick3(L.ox, L.oy, L.oz, kv);
    const float nd = frcp(fadd(fadd(dk, fmul(a0.y, du)), fmul(a0.z, dv)));
    return fmul(nd, fsub(fsub(fsub(a0.w, ok), fmul(a0.y, ou)), fmul(a0.z, ov)));
}

// The one-lane walk's test (the same decisions as test_tri).  A candidate
// that Moller-Trumbore puts clearly inside the triangle -- every barycentric
// at least kMtBarySlack inside, t at least the t slack inside the window,
// below the best so far and (any-hit) away from tmax -- is one the
// reference's test accepts too (both tests' errors stay far inside those
// margins), so it is accepted at once with Moller-Trumbore's t as the best
// so far (`fast_best`); only the candidates near an edge or a bound go to the
// reference's test, after the best so far has been replaced by its exact
// value.  The walk ends at the first cell with a hit, so a fast best never
// outlives its cell's list, and the reported values are recomputed exactly
// from the winner's record.
template <int MODE>
__device__ __forceinline__ bool test_tri_fast(Lane& L, int32_t tid, const float4& A, const float4& B,
                                              const float4& C, float hi, const float4* __restrict__ wald,
                                              bool& fast_best) {
#if GRIDRT_DECIDE_WALD
    const float tvx = L.ox - A.x, tvy = L.oy - A.y, tvz = L.oz - A.z;
    const float px = L.dy * C.z - L.dz * C.y;
    const float py = L.dz * C.x - L.dx * C.z;
    const float pz = L.dx * C.y - L.dy * C.x;
    const float det = B.x * px + B.y * py + B.z * pz;
    float idet;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(idet) : "f"(det));
    const float u = (tvx * px + tvy * py + tvz * pz) * idet;
    if (!(u >= -kMtBarySlack)) return false;
    const float qx = tvy * B.z - tvz * B.y;
    const float qy = tvz * B.x - tvx * B.z;
    const float qz = tvx * B.y - tvy * B.x;
    const float v = (L.dx * qx + L.dy * qy + L.dz * qz) * idet;
    const float w = (1.0f - u) - v;
    if (!(v >= -kMtBarySlack && w >= -kMtBarySlack)) return false;
    const float t = (C.x * qx + C.y * qy + C.z * qz) * idet;
    const float ts = fabsf(t) * kMtTRelSlack + kHitEpsilon;
    if (!((t < L.best + ts) && (t >= L.lo - ts) && (t <= hi + ts))) return false;
    const bool any_phase = MODE == MODE_ANY || (MODE == MODE_FRAME && L.tmax > -kFltMax);
    if (u >= kMtBarySlack && v >= kMtBarySlack && w >= kMtBarySlack && t >= L.lo + ts && t <= hi - ts &&
        t < L.best - ts && (!any_phase || t < L.tmax - ts || t > L.tmax + ts)) {
        L.best = t;
        L.id = tid;
        fast_best = true;
        return any_phase && t < L.tmax;
    }
    if (fast_best) {
        L.best = wald_f_of(L, L.id, wald);
        fast_best = false;
    }
    return wald_decide<MODE>(L, tid, hi, wald);
#else
    return test_tri<MODE>(L, tid, A, B, C, hi, wald);
#endif
}

// Visits up to ER empty cells and at most one non-empty cell.
// Returns true when the ray is finished (hit decided, or left the grid).
template <int MODE, int ER>
__device__ __forceinline__ bool advance(const SParams& P, Lane& L, const int32_t* __restrict__ offsets,
                                        const int32_t* __restrict__ ids, const float4* __restrict__ tris,
                                        const float4* __restrict__ wald,
                                        const uint32_t* __restrict__ occ, const float4* __restrict__ crec,
                                        int32_t heavy, int32_t work_cap, uint32_t& cells, uint32_t& tests) {
    const int32_t nx = P.res[0], nxy = P.res[0] * P.res[1];
    for (int s = 0; s < ER; ++s) {
        ++cells;
        const int32_t w = (L.x >> 2) + (L.y >> 2) * P.bx + (L.z >> 1) * P.bxby;
        if (w != L.cw) {
            L.cw = w;
            L.cword = __ldg(occ + w);
        }
        if (L.cword & occ_bit(L.x, L.y, L.z)) {
            const int32_t c = L.x + L.y * nx + L.z * nxy;
            const int32_t b = __ldg(offsets + c), e = __ldg(offsets + c + 1);
            if (e - b > heavy || L.work > work_cap - (e - b)) {
                // a long list, or a ray that has made many tests already
                // (grazing a surface): the ray goes to the deferred pass,
                // which resumes the walk at this cell (and counts it)
                --cells;
                L.id = kDeferred;
                return true;
            }
            L.work += e - b;
            const float hi = fadd(vmin(vmin(L.tMx, L.tMy), L.tMz), kHitEpsilon);
            tests += (uint32_t)(e - b);
            bool fast_best = false;
            int32_t i = b;
            if (crec) {
                // records stored in cell-list order: no id indirection
                for (; i + 1 < e; i += 2) {
                    const float4 A0 = __ldg(crec + 3 * (int64_t)i), B0 = __ldg(crec + 3 * (int64_t)i + 1),
                                 C0 = __ldg(crec + 3 * (int64_t)i + 2);
                    const float4 A1 = __ldg(crec + 3 * (int64_t)i + 3), B1 = __ldg(crec + 3 * (int64_t)i + 4),
                                 C1 = __ldg(crec + 3 * (int64_t)i + 5);
                    if (test_tri_fast<MODE>(L, __float_as_int(A0.w), A0, B0, C0, hi, wald, fast_best)) return true;
                    if (test_tri_fast<MODE>(L, __float_as_int(A1.w), A1, B1, C1, hi, wald, fast_best)) return true;
                }
                if (i < e) {
                    const float4 A0 = __ldg(crec + 3 * (int64_t)i), B0 = __ldg(crec + 3 * (int64_t)i + 1),
                                 C0 = __ldg(crec + 3 * (int64_t)i + 2);
                    if (test_tri_fast<MODE>(L, __float_as_int(A0.w), A0, B0, C0, hi, wald, fast_best)) return true;
                }
                i = e;
            }
            for (; i + 1 < e; i += 2) {
                const int32_t t0 = __ldg(ids + i), t1 = __ldg(ids + i + 1);
                const float4 A0 = __ldg(tris + 3 * (int64_t)t0), B0 = __ldg(tris + 3 * (int64_t)t0 + 1),
                             C0 = __ldg(tris + 3 * (int64_t)t0 + 2);
                const float4 A1 = __ldg(tris + 3 * (int64_t)t1), B1 = __ldg(tris + 3 * (int64_t)t1 + 1),
                             C1 = __ldg(tris + 3 * (int64_t)t1 + 2);
                if (test_tri_fast<MODE>(L, t0, A0, B0, C0, hi, wald, fast_best)) return true;
                if (test_tri_fast<MODE>(L, t1, A1, B1, C1, hi, wald, fast_best)) return true;
            }
            if (i < e) {
                const int32_t t0 = __ldg(ids + i);
                const float4 A0 = __ldg(tris + 3 * (int64_t)t0), B0 = __ldg(tris + 3 * (int64_t)t0 + 1),
                             C0 = __ldg(tris + 3 * (int64_t)t0 + 2);
                if (test_tri_fast<MODE>(L, t0, A0, B0, C0, hi, wald, fast_best)) return true;
            }
            if (L.id >= 0) {
                // a hit closer than the best on entry (the one-geometry walk
                // starts from FLT_MAX; an instance walk from the instances
                // before it).  Any-hit: the first cell with a hit decides --
                // here not before tmax
                if (MODE == MODE_ANY || (MODE == MODE_FRAME && L.tmax > -kFltMax)) L.id = -1;
                return true;
            }
            if (dda_step(P, L)) {
                L.id = -1;
                return true;
            }
            return false;
        }
        if (dda_step(P, L)) {
            L.id = -1;
            return true;
        }
    }
    return false;
}

// Reported hit values of the winning triangle: RayTriIntersection::hitWald
// (src/rtcore/RayTriIntersection.cpp:12-48) on the triangle's TriAccel record
// (written by the build exactly as TriAccel::buildFrom computes it), with the
// reference's operation order and one rounding per operation.  The accept /
// reject decisions of the walk stay Moller-Trumbore's; when the walk's winner
// is the reference's triangle, t (hitWald's f), u (lambda) and v (mue) are the
// reference's bits.
__device__ __forceinline__ int4 wald_hit(const float4* __restrict__ wald, const Lane& L) {
    const float4 a0 = __ldg(wald + 3 * (int64_t)L.id);
    const float4 a1 = __ldg(wald + 3 * (int64_t)L.id + 1);
    const float4 a2 = __ldg(wald + 3 * (int64_t)L.id + 2);
    const uint32_t k = __float_as_uint(a0.x);
    const uint32_t ku = k == 2 ? 0 : k + 1, kv = k == 0 ? 2 : k - 1;
    const float dk = pick3(L.dx, L.dy, L.dz, k), du = pick3(L.dx, L.dy, L.dz, ku), dv = pick3(L.dx, L.dy, L.dz, kv);
    const float ok = pick3(L.ox, L.oy, L.oz, k), ou = pick3(L.ox, L.oy, L.oz, ku), ov = pick3(L.ox, L.oy, L.oz, kv);
    const float nd = frcp(fadd(fadd(dk, fmul(a0.y, du)), fmul(a0.z, dv)));
    const float f = fmul(nd, fsub(fsub(fsub(a0.w, ok), fmul(a0.y, ou)), fmul(a0.z, ov)));
    const float hu = fadd(ou, fmul(f, du));
    const float hv = fadd(ov, fmul(f, dv));
    float lambda = fadd(fadd(fmul(hu, a1.x), fmul(hv, a1.y)), a1.z);
    float mue = fadd(fadd(fmul(hu, a2.x), fmul(hv, a2.y)), a2.z);
    float t = f;
    if (!(isfinite(f) && isfinite(lambda) && isfinite(mue))) {
        // a triangle without a finite projection record (the reference drops
        // such triangles at ingest): keep the walk's t
        t = L.best;
        lambda = 0.0f;
        mue = 0.0f;
    }
    return make_int4(L.id, __float_as_int(t), __float_as_int(lambda), __float_as_int(mue));
}

__device__ __forceinline__ void ray_pixel(int32_t i, const CameraArgs& cam, int32_t& px, int32_t& py) {
    if (cam.order == 1) {
        const int32_t tile = i >> 6;
        const int32_t r = (int32_t)(i & 63);
        const int32_t tiles_x = cam.width >> 3;
        const int32_t tx = (int32_t)(tile % tiles_x), ty = (int32_t)(tile / tiles_x);
        px = tx * 8 + ((r & 1) | ((r >> 1) & 2) | ((r >> 2) & 4));
        py = ty * 8 + (((r >> 1) & 1) | ((r >> 2) & 2) | ((r >> 3) & 4));
    } else {
        px = (int32_t)(i % cam.width);
        py = (int32_t)(i / cam.width);
    }
}

struct TraceIO {
    const float4* rays;       // NEAREST / ANY
    int4* hits;               // NEAREST / CAMERA
    uint8_t* occ;             // ANY
    float4* shadow_rays;      // CAMERA (optional): shadow or diffuse secondary rays
    CameraArgs cam;           // CAMERA
    float3 light;
    int has_light;
    int diffuse;              // CAMERA: secondary = cosine-weighted diffuse ray
    unsigned long long seed;
    long long n;
    unsigned long long* counter;   // [0] ray claims, [1] deferred rays, [2] deferred claims
    TraceCounters* ctr;
    int2* defer;                   // deferred rays {ray index, cell it stopped at} (nullptr: no deferral)
    int32_t defer_cap;
    int32_t heavy;                 // lists longer than this are deferred (kNoHeavy: never)
    int32_t defer_base;            // added to a deferred ray's index (a batch task's first)
    int32_t refill;                // > 0: lane refill at this many idle lanes (trace_refill)
    int2* huge;                    // rays at a list above kHugeList, for the block pass (nullptr: none)
    int32_t huge_cap;
};

// Loads ray `r` into the lane; false when the ray ends at once (misses the
// grid, or ANY mode with no shadow ray).
template <int MODE>
__device__ __forceinline__ bool start_ray(const SParams& P, const TraceIO& io, Lane& L, int32_t r) {
    float tnear, tfar;
    if (MODE == MODE_FRAME) L.tmax = -INFINITY;   // the camera phase
    if (MODE == MODE_CAMERA || MODE == MODE_FRAME) {
        int32_t px, py;
        ray_pixel(r, io.cam, px, py);
        const float us = fmul(fadd(__int2float_rn(px), 0.5f), io.cam.inv_w);
        const float vs = fmul(fadd(__int2float_rn(py), 0.5f), io.cam.inv_h);
        L.ox = io.cam.eye[0]; L.oy = io.cam.eye[1]; L.oz = io.cam.eye[2];
        L.dx = fadd(fadd(io.cam.base[0], fmul(io.cam.nu[0], us)), fmul(io.cam.nv[0], vs));
        L.dy = fadd(fadd(io.cam.base[1], fmul(io.cam.nu[1], us)), fmul(io.cam.nv[1], vs));
        L.dz = fadd(fadd(io.cam.base[2], fmul(io.cam.nu[2], us)), fmul(io.cam.nv[2], vs));
        tnear = kRayEpsilon;
        tfar = kFltMax;
    } else {
        const float4 a = __ldg(io.rays + 2 * (int64_t)r), b = __ldg(io.rays + 2 * (int64_t)r + 1);
        L.ox = a.x; L.oy = a.y; L.oz = a.z;
        L.dx = b.x; L.dy = b.y; L.dz = b.z;
        tnear = a.w;
        tfar = b.w;
        if (MODE == MODE_ANY && tfar < 0.0f) {   // no shadow ray for this slot
            L.id = -2;
            return false;
        }
    }
    L.id = -1;
    L.best = kFltMax;
    if (P.failed) return false;
    const bool ok = setup_ray(P, L, tnear, tfar);
    if (MODE == MODE_FRAME) L.tmax = -INFINITY;
    return ok;
}

// splitmix64 finaliser: counter-based random bits for ray index `i`.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// Cosine-weighted direction about unit normal n (Malley's method: uniform
// disc sample lifted to the hemisphere), 24-bit uniforms from mix64.
__device__ __forceinline__ float3 cosine_dir(float nx, float ny, float nz, unsigned long long bits) {
    const float u1 = (float)(bits >> 40) * (1.0f / 16777216.0f);
    const float u2 = (float)((bits >> 16) & 0xffffffull) * (1.0f / 16777216.0f);
    const float r = sqrtf(u1);
    float sp, cp;
    sincospif(2.0f * u2, &sp, &cp);
    const float lx = r * cp, ly = r * sp, lz = sqrtf(fmaxf(0.0f, 1.0f - u1));
    // orthonormal basis (Frisvad-style, branch on the sign of nz)
    const float sgn = nz >= 0.0f ? 1.0f : -1.0f;
    const float a = -1.0f / (sgn + nz);
    const float b = nx * ny * a;
    const float tx = 1.0f + sgn * nx * nx * a, ty = sgn * b, tz = -sgn * nx;
    const float bx = b, by = sgn + ny * ny * a, bz = -ny;
    return make_float3(lx * tx + ly * bx + lz * nx, lx * ty + ly * by + lz * ny, lx * tz + ly * bz + lz * nz);
}

// Writes the lane's result (when `write`: the lanes of a group or block that
// share a ray all compute it, one writes).  Returns true when the lane goes
// on with a follow-up ray: MODE_FRAME's camera phase sets up the hit's shadow
// ray in the lane, from the same values it writes to the shadow-ray slot.
template <int MODE>
__device__ __forceinline__ bool finish_ray(const TraceIO& io, const SParams& P, const SceneView& sv, Lane& L,
                                           bool write = true) {
    const float4* __restrict__ tris = sv.tris;
    const float4* __restrict__ wald = sv.wald;
    const int64_t r = L.ray;
    if (MODE == MODE_ANY || (MODE == MODE_FRAME && L.tmax > -kFltMax)) {
        if (write) io.occ[r] = L.id == -2 ? 2 : (L.id >= 0 ? 1 : 0);
        return false;
    }
    int4 h = make_int4(-1, 0, 0, 0);
    if (L.id >= 0) h = wald_hit(wald, L);
    if (write) io.hits[r] = h;
    if (MODE == MODE_CAMERA || MODE == MODE_FRAME) {
        float4 sa = make_float4(0.f, 0.f, 0.f, kRayEpsilon), sb = make_float4(0.f, 0.f, 0.f, -1.0f);
        if (L.id >= 0 && io.diffuse) {
            // secondary diffuse ray from the hit point, offset along the
            // normal facing the incoming ray, tnear 2e-4, tfar FLT_MAX
            const float t = __int_as_float(h.y);
            const float4 B = __ldg(tris + 3 * (int64_t)L.id + 1);
            const float4 C = __ldg(tris + 3 * (int64_t)L.id + 2);
            float nx = B.y * C.z - B.z * C.y, ny = B.z * C.x - B.x * C.z, nz = B.x * C.y - B.y * C.x;
            const float rl = rsqrtf(nx * nx + ny * ny + nz * nz);
            nx *= rl; ny *= rl; nz *= rl;
            if (nx * L.dx + ny * L.dy + nz * L.dz > 0.0f) { nx = -nx; ny = -ny; nz = -nz; }
            const float3 w = cosine_dir(nx, ny, nz, mix64(io.seed ^ mix64((unsigned long long)r)));
            sa = make_float4(L.ox + L.dx * t + nx * kRayEpsilon, L.oy + L.dy * t + ny * kRayEpsilon,
                             L.oz + L.dz * t + nz * kRayEpsilon, kRayEpsilon);
            sb = make_float4(w.x, w.y, w.z, kFltMax);
        } else if (L.id >= 0 && io.has_light) {
            // Sample::computeHitPosition, flat normal facing the ray, initLightRay
            // offset and initShadowRay (src/rtcore/Sample.cpp:22-42,177-180,224-236),
            // SimplePointLight::illuminate (src/rtplugins/SimplePointLight.cpp:25-33)
            const float t = __int_as_float(h.y);
            const float4 B = __ldg(tris + 3 * (int64_t)L.id + 1);
            const float4 C = __ldg(tris + 3 * (int64_t)L.id + 2);
            float nx = B.y * C.z - B.z * C.y, ny = B.z * C.x - B.x * C.z, nz = B.x * C.y - B.y * C.x;
            const float rl = rsqrtf(nx * nx + ny * ny + nz * nz);
            nx *= rl; ny *= rl; nz *= rl;
            if (nx * L.dx + ny * L.dy + nz * L.dz > 0.0f) { nx = -nx; ny = -ny; nz = -nz; }
            const float hx = L.ox + L.dx * t + nx * kRayEpsilon;
            const float hy = L.oy + L.dy * t + ny * kRayEpsilon;
            const float hz = L.oz + L.dz * t + nz * kRayEpsilon;
            const float lx = io.light.x - hx, ly = io.light.y - hy, lz = io.light.z - hz;
            if (nx * lx + ny * ly + nz * lz > 0.0f) {
                sa = make_float4(hx, hy, hz, kRayEpsilon);
                sb = make_float4(lx, ly, lz, 1.0f);
            }
        }
        if (io.shadow_rays && write) {
            io.shadow_rays[2 * r] = sa;
            io.shadow_rays[2 * r + 1] = sb;
        }
        if (MODE == MODE_FRAME) {
            // the shadow ray as the any-hit pass would load it from the slot
            if (sb.w < 0.0f) {
                if (write) io.occ[r] = 2;
                return false;
            }
            L.ox = sa.x; L.oy = sa.y; L.oz = sa.z;
            L.dx = sb.x; L.dy = sb.y; L.dz = sb.z;
            L.id = -1;
            L.best = kFltMax;
            if (!setup_ray(P, L, sa.w, sb.w)) {
                if (write) io.occ[r] = 0;
                return false;
            }
            return true;
        }
    }
    return false;
}

// Deferred-queue entry of the lane's ray: its index (plus a batch task's
// first), or -1 - index for a MODE_FRAME shadow ray.
template <int MODE>
__device__ __forceinline__ int32_t defer_tag(const Lane& L, const TraceIO& io) {
    return (MODE == MODE_FRAME && L.tmax > -kFltMax) ? -1 - L.ray : L.ray + io.defer_base;
}

template <int MODE, int ER>
__device__ __forceinline__ void trace_batch32(const SParams& P, const SceneView& s, const TraceIO& io, Lane& L,
                                              long long base, uint32_t& cells, uint32_t& tests, uint32_t& started) {
    const int lane = threadIdx.x & 31;
    const long long ray = base + lane;
    bool active = ray < io.n;
    L.ray = (int32_t)ray;
    int32_t heavy = io.heavy;
    int32_t work_cap = heavy < kNoHeavy / (kHeavyWorkMult + 1) && kHeavyWorkMult > 0 ? heavy * kHeavyWorkMult
                                                                                    : kNoHeavy;
    if (active) {
        ++started;
        if (!start_ray<MODE>(P, io, L, L.ray)) {
            if (L.id != -2) L.id = -1;
            active = finish_ray<MODE>(io, P, s, L);
        }
    }
    while (__any_sync(FULL, active)) {
        bool fin = active &&
                   advance<MODE, ER>(P, L, s.offsets, s.ids, s.tris, s.wald, s.occ, s.crec, heavy, work_cap, cells, tests);
        if (io.defer) {
            // warp-aggregated push of the lanes that met a long list
            const bool d = fin && L.id == kDeferred;
            const unsigned m = __ballot_sync(FULL, d);
            if (m) {
                const int leader = __ffs(m) - 1;
                unsigned long long at = 0;
                if (lane == leader) at = atomicAdd(io.counter + 1, (unsigned long long)__popc(m));
                at = __shfl_sync(FULL, at, leader);
                if (d) {
                    const unsigned long long slot = at + __popc(m & ((1u << lane) - 1u));
                    if (slot < (unsigned long long)io.defer_cap) {
                        // the walk resumes at this cell in the warp-per-ray pass
                        io.defer[slot] = make_int2(defer_tag<MODE>(L, io), L.x + L.y * P.res[0] + L.z * P.res[0] * P.res[1]);
                        active = false;
                    } else {
                        heavy = kNoHeavy;        // queue full: the lane tests the cell itself
                        work_cap = kNoHeavy;
                        L.id = -1;
                    }
                    fin = false;
                }
            }
        }
        if (fin) active = finish_ray<MODE>(io, P, s, L);
    }
}

__device__ __forceinline__ void flush_counters(TraceCounters* ctr, uint32_t started, uint32_t cells, uint32_t tests) {
    unsigned long long r = started, c = cells, t = tests;
    for (int o = 16; o > 0; o >>= 1) {
        r += __shfl_xor_sync(FULL, r, o);
        c += __shfl_xor_sync(FULL, c, o);
        t += __shfl_xor_sync(FULL, t, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&ctr->rays, r);
        atomicAdd(&ctr->cells, c);
        atomicAdd(&ctr->tests, t);
    }
}

// Eight blocks of 128 threads per SM (64 registers a thread): the walk is
// latency-bound, and resident warps matter more than the few spilled words.
#ifndef GRIDRT_TRACE_MIN_BLOCKS
#define GRIDRT_TRACE_MIN_BLOCKS 8
#endif

// Lane refill (TraceIO::refill > 0): instead of tracing a claimed batch of
// 32 rays to its end, the warp hands new rays to its idle lanes whenever at
// least `refill` of them are idle (one claim for all of them), keeping the
// lanes busy while long rays finish.  Pays on incoherent rays, whose walks
// differ most in length (diffuse secondaries: -11% trace time); costs ~2% on
// coherent camera rays, so it is a tuning choice.
template <int MODE, int ER>
__device__ __forceinline__ void trace_refill(const SParams& P, const SceneView& s, const TraceIO& io, Lane& L,
                                             uint32_t& cells, uint32_t& tests, uint32_t& started) {
    const int lane = threadIdx.x & 31;
    bool active = false, exhausted = false;
    int32_t heavy = io.heavy, work_cap = kNoHeavy;
    for (;;) {
        const unsigned idle = __ballot_sync(FULL, !active);
        if (!exhausted && ((int)__popc(idle) >= io.refill || idle == FULL)) {
            const unsigned need = (unsigned)__popc(idle);
            unsigned long long b = 0;
            if (lane == 0) b = atomicAdd(io.counter, (unsigned long long)need);
            b = __shfl_sync(FULL, b, 0);
            if ((long long)(b + need) >= io.n) exhausted = true;
            if (!active) {
                const long long ray = (long long)b + __popc(idle & ((1u << lane) - 1u));
                if (ray < io.n) {
                    L.ray = (int32_t)ray;
                    heavy = io.heavy;
                    work_cap = heavy < kNoHeavy / (kHeavyWorkMult + 1) && kHeavyWorkMult > 0 ? heavy * kHeavyWorkMult
                                                                                             : kNoHeavy;
                    ++started;
                    if (start_ray<MODE>(P, io, L, L.ray)) {
                        active = true;
                    } else {
                        if (L.id != -2) L.id = -1;
                        active = finish_ray<MODE>(io, P, s, L);
                    }
                }
            }
        }
        if (!__any_sync(FULL, active)) {
            if (exhausted) break;
            continue;
        }
        bool fin = active &&
                   advance<MODE, ER>(P, L, s.offsets, s.ids, s.tris, s.wald, s.occ, s.crec, heavy, work_cap, cells, tests);
        if (io.defer) {
            const bool d = fin && L.id == kDeferred;
            const unsigned m = __ballot_sync(FULL, d);
            if (m) {
                const int leader = __ffs(m) - 1;
                unsigned long long at = 0;
                if (lane == leader) at = atomicAdd(io.counter + 1, (unsigned long long)__popc(m));
                at = __shfl_sync(FULL, at, leader);
                if (d) {
                    const unsigned long long slot = at + __popc(m & ((1u << lane) - 1u));
                    if (slot < (unsigned long long)io.defer_cap) {
                        io.defer[slot] = make_int2(defer_tag<MODE>(L, io),
                                                   L.x + L.y * P.res[0] + L.z * P.res[0] * P.res[1]);
                        active = false;
                    } else {
                        heavy = kNoHeavy;
                        work_cap = kNoHeavy;
                        L.id = -1;
                    }
                    fin = false;
                }
            }
        }
        if (fin) active = finish_ray<MODE>(io, P, s, L);
    }
}

template <int MODE, bool COUNT, int ER, int TPB>
__global__ void __launch_bounds__(TPB, GRIDRT_TRACE_MIN_BLOCKS * 128 / TPB) trace_kernel(SceneView s, TraceIO io) {
    pdl_begin();
    __shared__ SParams P;
    load_sparams(s.params, P);
    const int lane = threadIdx.x & 31;
    Lane L;
    uint32_t cells = 0, tests = 0, started = 0;
    if (io.refill > 0) {
        trace_refill<MODE, ER>(P, s, io, L, cells, tests, started);
    } else {
        for (;;) {
            // the warp claims the next 32 consecutive rays and traces them to the end
            unsigned long long b = 0;
            if (lane == 0) b = atomicAdd(io.counter, 32ull);
            b = __shfl_sync(FULL, b, 0);
            if ((long long)b >= io.n) break;
            trace_batch32<MODE, ER>(P, s, io, L, (long long)b, cells, tests, started);
        }
    }
    if (COUNT) flush_counters(io.ctr, started, cells, tests);
}

// Warp-per-ray pass over the deferred rays, G lanes per ray (32/G rays a
// warp): the G lanes of a group hold the same ray and walk the same cells; a
// cell's list is split over them (lane j of the group tests entries j, j+G,
// ...), each lane keeping the first minimum of its share, and the group
// takes the minimum t, ties to the smaller triangle id.  Lists are sorted by
// id, so that is the first minimum in list order: the one-lane walk's result.
// ANY rays are occluded when that minimum is below tmax -- also the one-lane
// walk's rule, which accepts every new minimum and stops at the first below
// tmax.
//
// A deferred ray resumes at the cell where its lane stopped: every coordinate
// moved monotonically from the start cell, one step per crossing of its
// axis, each adding tD to tM, so replaying those additions in order rebuilds
// the walk's exact state there (the earlier cells were tested without a hit).
__device__ __forceinline__ void resume_at(const SParams& P, Lane& L, int32_t cell) {
    const int32_t nx = P.res[0], nxy = P.res[0] * P.res[1];
    const int32_t z = cell / nxy, y = (cell - z * nxy) / nx, x = cell - z * nxy - y * nx;
    const int32_t sx = abs(x - L.x), sy = abs(y - L.y), sz = abs(z - L.z);
    for (int32_t i = 0; i < sx; ++i) L.tMx = fadd(L.tMx, L.tDx);
    for (int32_t i = 0; i < sy; ++i) L.tMy = fadd(L.tMy, L.tDy);
    for (int32_t i = 0; i < sz; ++i) L.tMz = fadd(L.tMz, L.tDz);
    L.x = x;
    L.y = y;
    L.z = z;
    L.budget -= sx + sy + sz;
}

// Walks the group's ray (state in L, identical on its G lanes) to its end.
// Every lane of the warp calls it; groups that are done idle through the
// warp-wide list loop and reductions.
// With `huge` set, a group whose ray reaches a list above kHugeList queues
// {huge_tag, cell} for the block-per-ray pass instead (counted there) and
// returns true: that pass finishes the ray.
template <int G>
__device__ __forceinline__ bool wide_walk(const SParams& P, const SceneView& s, Lane& L, bool done, bool any,
                                          uint32_t& cells, uint32_t& tests, int2* huge = nullptr,
                                          int32_t huge_cap = 0, unsigned long long* huge_ctr = nullptr,
                                          int32_t huge_tag = 0) {
    const int gl = threadIdx.x & (G - 1);
    bool handed = false;
    const int32_t nx = P.res[0], nxy = P.res[0] * P.res[1];
    while (__any_sync(FULL, !done)) {
        int32_t b = 0, e = 0;
        float hi = 0.0f;
        if (!done) {
            // up to kWideEmptyRun empty cells per turn before a list (as the
            // one-lane walk does), so empty stretches skip the list and
            // reduction steps below
            for (int r = 0; r < kWideEmptyRun; ++r) {
                if (gl == 0) ++cells;
                const int32_t w = (L.x >> 2) + (L.y >> 2) * P.bx + (L.z >> 1) * P.bxby;
                if (__ldg(s.occ + w) & occ_bit(L.x, L.y, L.z)) {
                    const int32_t c = L.x + L.y * nx + L.z * nxy;
                    b = __ldg(s.offsets + c);
                    e = __ldg(s.offsets + c + 1);
                    hi = fadd(vmin(vmin(L.tMx, L.tMy), L.tMz), kHitEpsilon);
                    break;
                }
                if (dda_step(P, L)) {
                    L.id = -1;
                    done = true;
                    break;
                }
            }
        }
        if (huge) {
            // lists above kHugeList go to the block-per-ray pass (which visits
            // the cell again), while its queue has room
            const bool want = !done && e - b > kHugeList;
            if (__ballot_sync(FULL, want)) {
                unsigned long long at = 0;
                if (want && gl == 0) at = atomicAdd(huge_ctr, 1ull);
                at = __shfl_sync(FULL, at, (int)(threadIdx.x & 31) & ~(G - 1));
                if (want && at < (unsigned long long)huge_cap) {
                    if (gl == 0) {
                        // longest first: lists of kHugeLong+ entries fill the
                        // queue from its back (huge_ctr[2] of them), the rest
                        // from its front (huge_ctr[3]); together they number
                        // the reservations that fit, so the two never meet
                        const bool longl = e - b >= kHugeLong;
                        const unsigned long long pos = atomicAdd(huge_ctr + (longl ? 2 : 3), 1ull);
                        huge[longl ? (unsigned long long)huge_cap - 1 - pos : pos] =
                            make_int2(huge_tag, L.x + L.y * nx + L.z * nxy);
                        --cells;
                    }
                    handed = done = true;
                    b = e = 0;
                }
            }
        }
        if (gl == 0) tests += (uint32_t)(e - b);
        const unsigned trips = __reduce_max_sync(FULL, (unsigned)((e - b + G - 1) / G));
        if (trips == 0) continue;   // no group of the warp is at a list this turn
        // two entries per lane and turn, both loaded before either is tested
        for (unsigned it = 0; it < trips; it += 2) {
            const int32_t i0 = b + gl + (int32_t)it * G, i1 = i0 + G;
            int32_t t0 = -1, t1 = -1;
            float4 A0, B0, C0, A1, B1, C1;
            if (s.crec) {
                if (i0 < e) {
                    A0 = __ldg(s.crec + 3 * (int64_t)i0);
                    B0 = __ldg(s.crec + 3 * (int64_t)i0 + 1);
                    C0 = __ldg(s.crec + 3 * (int64_t)i0 + 2);
                    t0 = __float_as_int(A0.w);
                }
                if (i1 < e) {
                    A1 = __ldg(s.crec + 3 * (int64_t)i1);
                    B1 = __ldg(s.crec + 3 * (int64_t)i1 + 1);
                    C1 = __ldg(s.crec + 3 * (int64_t)i1 + 2);
                    t1 = __float_as_int(A1.w);
                }
            } else {
                if (i0 < e) t0 = __ldg(s.ids + i0);
                if (i1 < e) t1 = __ldg(s.ids + i1);
                if (t0 >= 0) {
                    A0 = __ldg(s.tris + 3 * (int64_t)t0);
                    B0 = __ldg(s.tris + 3 * (int64_t)t0 + 1);
                    C0 = __ldg(s.tris + 3 * (int64_t)t0 + 2);
                }
                if (t1 >= 0) {
                    A1 = __ldg(s.tris + 3 * (int64_t)t1);
                    B1 = __ldg(s.tris + 3 * (int64_t)t1 + 1);
                    C1 = __ldg(s.tris + 3 * (int64_t)t1 + 2);
                }
            }
            if (t0 >= 0) test_tri<MODE_NEAREST>(L, t0, A0, B0, C0, hi, s.wald);
            if (t1 >= 0) test_tri<MODE_NEAREST>(L, t1, A1, B1, C1, hi, s.wald);
        }
#pragma unroll
        for (int o = G >> 1; o > 0; o >>= 1) {
            const float ot = __shfl_xor_sync(FULL, L.best, o);
            const int32_t oid = __shfl_xor_sync(FULL, L.id, o);
            if (ot < L.best || (ot == L.best && (uint32_t)oid < (uint32_t)L.id)) {
                L.best = ot;
                L.id = oid;
            }
        }
        if (!done && e > b) {   // groups that tested a list this turn
            if (L.best < kFltMax) {
                if (any && !(L.best < L.tmax)) L.id = -1;
                done = true;
            } else if (dda_step(P, L)) {
                L.id = -1;
                done = true;
            }
        }
    }
    return handed;
}

// Five blocks of 128 threads per SM (at most 102 registers a thread): the
// exact decisions' code took the group pass from 96 to 109 registers, four
// blocks an SM, and 20% longer.
#ifndef GRIDRT_WIDE_MIN_BLOCKS
#define GRIDRT_WIDE_MIN_BLOCKS 5
#endif
template <int MODE, bool COUNT, int G>
__global__ void __launch_bounds__(128, GRIDRT_WIDE_MIN_BLOCKS) trace_wide_kernel(SceneView s, TraceIO io) {
    pdl_begin();
    __shared__ SParams P;
    load_sparams(s.params, P);
    const int lane = threadIdx.x & 31, gl = lane & (G - 1), grp = lane / G;
    // the deferred rays, or (no queue: the group walk from the start) every ray
    unsigned long long nd = io.defer ? io.counter[1] : (unsigned long long)io.n;
    if (io.defer && nd > (unsigned long long)io.defer_cap) nd = (unsigned long long)io.defer_cap;
    uint32_t cells = 0, tests = 0;
    for (;;) {
        unsigned long long j0 = 0;
        if (lane == 0) j0 = atomicAdd(io.counter + 2, (unsigned long long)(32 / G));
        j0 = __shfl_sync(FULL, j0, 0);
        if (j0 >= nd) break;
        const unsigned long long j = j0 + grp;
        const bool valid = j < nd;
        bool done = true;
        Lane L;
        L.best = kFltMax;
        L.id = -1;
        bool shadow = false;      // MODE_FRAME: the entry is a shadow ray (its slot holds it)
        if (valid) {
            const int2 d = io.defer ? __ldg(io.defer + j) : make_int2((int32_t)j, -1);
            shadow = MODE == MODE_FRAME && d.x < 0;
            L.ray = shadow ? -1 - d.x : d.x;
            done = shadow ? !start_ray<MODE_ANY>(P, io, L, L.ray) : !start_ray<MODE>(P, io, L, L.ray);
            if (done) {
                if (L.id != -2) L.id = -1;
            } else if (d.y >= 0) {
                resume_at(P, L, d.y);
            }
        }
        const bool handed = wide_walk<G>(P, s, L, done, MODE == MODE_ANY || shadow, cells, tests, io.huge,
                                         io.huge_cap, io.counter + 3, shadow ? -1 - L.ray : L.ray);
        if (MODE == MODE_FRAME) {
            // a camera ray's group goes on with its hit's shadow ray: every
            // lane sets it up from the hit (one writes the results)
            bool second = false;
            if (valid && !handed) second = finish_ray<MODE>(io, P, s, L, gl == 0);
            bool done2 = !second;
            const bool handed2 = wide_walk<G>(P, s, L, done2, true, cells, tests, io.huge, io.huge_cap,
                                              io.counter + 3, -1 - L.ray);
            if (second && !handed2 && gl == 0) finish_ray<MODE>(io, P, s, L);
        } else if (valid && gl == 0 && !handed) {
            finish_ray<MODE>(io, P, s, L);
        }
    }
    if (COUNT) {
        if (gl != 0) cells = tests = 0;
        flush_counters(io.ctr, 0, cells, tests);
    }
}

// Block-per-ray pass over the rays the group pass met at a list above
// kHugeList (a dense cluster: tens of thousands of triangles in one cell):
// all threads of the block hold the ray and step the same DDA; each list is
// split over the block (thread j tests entries j, j + blockDim, ...), each
// thread keeping the first minimum of its share, and a block reduction takes
// the minimum t, ties to the earlier entry -- the one-lane walk's result, as
// in the group pass.  A ray's walk then takes a block's time per list, not a
// lane's or a group's.
#ifndef GRIDRT_HUGE_THREADS
#define GRIDRT_HUGE_THREADS 256
#endif
static constexpr int kHugeThreads = GRIDRT_HUGE_THREADS;
#ifndef GRIDRT_HUGE_MIN_BLOCKS
#define GRIDRT_HUGE_MIN_BLOCKS 3
#endif
static_assert(kHugeThreads % 32 == 0 && kHugeThreads <= 1024, "block-per-ray pass: whole warps, one block");

// Crowded lists staged in shared memory.  With cell-ordered records a list
// is one contiguous run of 48-byte records, so the bulk-copy engine
// (cp.async.bulk, completion counted on an mbarrier per buffer) copies it
// into a ring of kStageDepth shared-memory buffers of kStageEntries records:
// while the block tests one chunk the next kStageDepth - 1 are in flight,
// and no thread waits on its own global loads.  A chunk costs a block
// barrier and a wait, so chunks are large: 768 records (36 KB), two
// buffers, 72 KB a block and three blocks an SM (smaller chunks or deeper
// rings measured slower).  Lists shorter than kStageMin keep the direct
// loads.  Every wait is bounded: a copy that has not landed after
// kStageWaitLimit polls sets bit 0 of the launch's counter word 7, the rest
// of the list is tested from global memory and the block stops staging.
#ifndef GRIDRT_STAGE
#define GRIDRT_STAGE 1
#endif
#ifndef GRIDRT_STAGE_ENTRIES
#define GRIDRT_STAGE_ENTRIES 768
#endif
#ifndef GRIDRT_STAGE_DEPTH
#define GRIDRT_STAGE_DEPTH 2
#endif
static constexpr int kStageEntries = GRIDRT_STAGE_ENTRIES;
static constexpr int kStageDepth = GRIDRT_STAGE_DEPTH;
static constexpr size_t kStageBytes = GRIDRT_STAGE ? (size_t)kStageDepth * 3 * kStageEntries * sizeof(float4) : 0;
static_assert(kStageDepth >= 2 && kStageDepth <= 16, "stage ring depth");
static constexpr int32_t kStageMin = 2 * kHugeThreads;
static constexpr uint32_t kStageWaitLimit = 1u << 24;
static_assert(kStageEntries % kHugeThreads == 0 || kHugeThreads % kStageEntries == 0, "stage chunk");

struct Stage {
    float4* buf;          // shared: kStageDepth x kStageEntries x 3 float4
    uint64_t* bar;        // shared: one mbarrier per buffer
    int* off;             // shared: 1 once a wait has run out
    uint32_t phase;       // bit q: the parity of buffer q's next completion
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Thread 0: buffer `dst` <- `bytes` of global memory at `src`, completion
// on `bar` (which expects those bytes and thread 0's arrival).
__device__ __forceinline__ void stage_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Bounded wait for the completion of `bar`'s phase of parity `parity`.
__device__ __forceinline__ bool stage_wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t it = 0; it < kStageWaitLimit; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// The block's ray (identical state on every thread) walked to its end:
// each list split over the block, a block reduction per list.
__device__ __forceinline__ void block_walk(const SParams& P, const SceneView& s, Lane& L, bool done, bool any,
                                           uint32_t& cells, uint32_t& tests, float* red_t, int32_t* red_id,
                                           Stage* st = nullptr, unsigned long long* err = nullptr) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int32_t nx = P.res[0], nxy = P.res[0] * P.res[1];
    while (!done) {
        if (threadIdx.x == 0) ++cells;
        const int32_t w = (L.x >> 2) + (L.y >> 2) * P.bx + (L.z >> 1) * P.bxby;
        if (__ldg(s.occ + w) & occ_bit(L.x, L.y, L.z)) {
            const int32_t c = L.x + L.y * nx + L.z * nxy;
            const int32_t b = __ldg(s.offsets + c), e = __ldg(s.offsets + c + 1);
            const float hi = fadd(vmin(vmin(L.tMx, L.tMy), L.tMz), kHitEpsilon);
            if (threadIdx.x == 0) tests += (uint32_t)(e - b);
            Lane T = L;
            T.id = -1;
            if (GRIDRT_STAGE && st && s.crec && e - b >= kStageMin && !*st->off) {
                // staged: chunk ch in buffer ch % kStageDepth, the next
                // kStageDepth - 1 chunks in flight
                const int32_t nch = (e - b + kStageEntries - 1) / kStageEntries;
                if (threadIdx.x == 0) {
                    for (int32_t ch = 0; ch < nch && ch < kStageDepth; ++ch) {
                        const int32_t cb = b + ch * kStageEntries;
                        const int32_t cn = e - cb < kStageEntries ? e - cb : kStageEntries;
                        stage_copy(st->buf + ch * 3 * kStageEntries, s.crec + 3 * (int64_t)cb, (uint32_t)cn * 48u,
                                   st->bar + ch);
                    }
                }
                for (int32_t ch = 0; ch < nch; ++ch) {
                    const int q = ch % kStageDepth;
                    const int32_t cb = b + ch * kStageEntries;
                    const int32_t cn = e - cb < kStageEntries ? e - cb : kStageEntries;
                    const bool ok = stage_wait(st->bar + q, (st->phase >> q) & 1u);
                    st->phase ^= 1u << q;
                    if (ok) {
                        const float4* sb = st->buf + q * 3 * kStageEntries;
                        for (int32_t j = (int32_t)threadIdx.x; j < cn; j += kHugeThreads) {
                            const float4 A = sb[3 * j], B = sb[3 * j + 1], C = sb[3 * j + 2];
                            test_tri<MODE_NEAREST>(T, __float_as_int(A.w), A, B, C, hi, s.wald);
                        }
                    }
                    // every thread is done with buffer q before chunk
                    // ch + kStageDepth is copied into it
                    if (__syncthreads_or(!ok)) {
                        // a copy has not landed: wait once more (bounded) for
                        // it and the copies in flight behind it, test the rest
                        // of the list from global memory, stop staging
                        if (!ok) stage_wait(st->bar + q, ((st->phase >> q) & 1u) ^ 1u);
                        for (int32_t k = ch + 1; k < nch && k < ch + kStageDepth; ++k) {
                            const int qk = k % kStageDepth;
                            stage_wait(st->bar + qk, (st->phase >> qk) & 1u);
                        }
                        if (threadIdx.x == 0) {
                            *st->off = 1;
                            if (err) atomicOr(err, 1ull);
                        }
                        for (int32_t i = (ok ? cb + cn : cb) + (int32_t)threadIdx.x; i < e; i += kHugeThreads) {
                            const float4 A = __ldg(s.crec + 3 * (int64_t)i), B = __ldg(s.crec + 3 * (int64_t)i + 1),
                                         C = __ldg(s.crec + 3 * (int64_t)i + 2);
                            test_tri<MODE_NEAREST>(T, __float_as_int(A.w), A, B, C, hi, s.wald);
                        }
                        __syncthreads();
                        break;
                    }
                    if (threadIdx.x == 0 && ch + kStageDepth < nch) {
                        const int32_t nb = cb + kStageDepth * kStageEntries;
                        const int32_t nn = e - nb < kStageEntries ? e - nb : kStageEntries;
                        stage_copy(st->buf + q * 3 * kStageEntries, s.crec + 3 * (int64_t)nb, (uint32_t)nn * 48u,
                                   st->bar + q);
                    }
                }
            } else if (s.crec) {
                // two entries a thread per step, both loaded before either is
                // tested (the same entries in the same order as one a step)
                for (int32_t i = b + (int32_t)threadIdx.x; i < e; i += 2 * kHugeThreads) {
                    const int32_t i2 = i + kHugeThreads;
                    const float4 A = __ldg(s.crec + 3 * (int64_t)i), B = __ldg(s.crec + 3 * (int64_t)i + 1),
                                 C = __ldg(s.crec + 3 * (int64_t)i + 2);
                    float4 A2 = A, B2 = B, C2 = C;
                    if (i2 < e) {
                        A2 = __ldg(s.crec + 3 * (int64_t)i2);
                        B2 = __ldg(s.crec + 3 * (int64_t)i2 + 1);
                        C2 = __ldg(s.crec + 3 * (int64_t)i2 + 2);
                    }
                    test_tri<MODE_NEAREST>(T, __float_as_int(A.w), A, B, C, hi, s.wald);
                    if (i2 < e) test_tri<MODE_NEAREST>(T, __float_as_int(A2.w), A2, B2, C2, hi, s.wald);
                }
            } else {
                for (int32_t i = b + (int32_t)threadIdx.x; i < e; i += 2 * kHugeThreads) {
                    const int32_t i2 = i + kHugeThreads;
                    const int32_t t = __ldg(s.ids + i), t2 = i2 < e ? __ldg(s.ids + i2) : t;
                    const float4 A = __ldg(s.tris + 3 * (int64_t)t), B = __ldg(s.tris + 3 * (int64_t)t + 1),
                                 C = __ldg(s.tris + 3 * (int64_t)t + 2);
                    const float4 A2 = __ldg(s.tris + 3 * (int64_t)t2), B2 = __ldg(s.tris + 3 * (int64_t)t2 + 1),
                                 C2 = __ldg(s.tris + 3 * (int64_t)t2 + 2);
                    test_tri<MODE_NEAREST>(T, t, A, B, C, hi, s.wald);
                    if (i2 < e) test_tri<MODE_NEAREST>(T, t2, A2, B2, C2, hi, s.wald);
                }
            }
            // ids ascend along a list: the smaller id is the earlier entry
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float ot = __shfl_xor_sync(FULL, T.best, o);
                const int32_t oid = __shfl_xor_sync(FULL, T.id, o);
                if (ot < T.best || (ot == T.best && (uint32_t)oid < (uint32_t)T.id)) {
                    T.best = ot;
                    T.id = oid;
                }
            }
            if (lane == 0) {
                red_t[wid] = T.best;
                red_id[wid] = T.id;
            }
            __syncthreads();
            float bt = red_t[0];
            int32_t bid = red_id[0];
            for (int i = 1; i < kHugeThreads / 32; ++i)
                if (red_t[i] < bt || (red_t[i] == bt && (uint32_t)red_id[i] < (uint32_t)bid)) {
                    bt = red_t[i];
                    bid = red_id[i];
                }
            __syncthreads();
            if (bid >= 0) {
                // the first cell with a hit ends the walk; any-hit:
                // occluded only below tmax
                L.best = bt;
                L.id = (any && !(bt < L.tmax)) ? -1 : bid;
                done = true;
                continue;
            }
        }
        if (dda_step(P, L)) {
            L.id = -1;
            done = true;
        }
    }
}

template <int MODE, bool COUNT>
__global__ void __launch_bounds__(kHugeThreads, GRIDRT_HUGE_MIN_BLOCKS) trace_huge_kernel(SceneView s, TraceIO io) {
    pdl_begin();
    __shared__ SParams P;
    __shared__ float red_t[kHugeThreads / 32];
    __shared__ int32_t red_id[kHugeThreads / 32];
    __shared__ unsigned long long claim;
    extern __shared__ __align__(128) float4 stage_buf[];   // kStageBytes (dynamic)
    __shared__ __align__(8) uint64_t stage_bar[kStageDepth];
    __shared__ int stage_off;
    if (threadIdx.x == 0) {
        for (int q = 0; q < kStageDepth; ++q)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(stage_bar + q)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        stage_off = 0;
    }
    Stage stage{stage_buf, stage_bar, &stage_off, 0u};
    load_sparams(s.params, P);
    unsigned long long nh = io.counter[3];
    if (nh > (unsigned long long)io.huge_cap) nh = (unsigned long long)io.huge_cap;
    // the rays at the longest lists (the queue's back) are claimed first, so
    // they do not start last and run on alone at the end of the pass
    const unsigned long long nb = io.counter[5];
    uint32_t cells = 0, tests = 0;
    for (;;) {
        if (threadIdx.x == 0) claim = atomicAdd(io.counter + 4, 1ull);
        __syncthreads();
        const unsigned long long j = claim;
        __syncthreads();
        if (j >= nh) break;
        const int2 d = __ldg(io.huge + (j < nb ? (unsigned long long)io.huge_cap - 1 - j : j - nb));
        const bool shadow = MODE == MODE_FRAME && d.x < 0;   // MODE_FRAME: a shadow ray (in its slot)
        Lane L;
        L.ray = shadow ? -1 - d.x : d.x;
        // the same on every thread
        bool done = shadow ? !start_ray<MODE_ANY>(P, io, L, L.ray) : !start_ray<MODE>(P, io, L, L.ray);
        if (done) {
            if (L.id != -2) L.id = -1;
        } else {
            resume_at(P, L, d.y);
        }
        // one walk, or for a MODE_FRAME camera ray two: its own, then from
        // its start the shadow ray every thread sets up from the hit
        for (int phase = 0; phase < 2; ++phase) {
            block_walk(P, s, L, done, MODE == MODE_ANY || (MODE == MODE_FRAME && L.tmax > -kFltMax), cells, tests,
                       red_t, red_id, &stage, io.counter + 7);
            if (!finish_ray<MODE>(io, P, s, L, threadIdx.x == 0)) break;
            done = false;
        }
    }
    if (COUNT) {
        if (threadIdx.x != 0) cells = tests = 0;
        flush_counters(io.ctr, 0, cells, tests);
    }
}

// Blocks of TPB threads (the RTG_TUNE_BLOCK choice; counter launches use
// 128).  Persistent: as many blocks as fit on the device at once, warps loop
// over ray batches.  One-shot: one batch per warp, blocks scheduled by the
// hardware.
template <int MODE, bool COUNT, int ER, int TPB>
inline void launch_tpb(const SceneView& s, const TraceIO& io, const TraceTuning& tune, int num_sms, cudaStream_t st) {
    static int per_sm = 0;
    if (per_sm == 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, trace_kernel<MODE, COUNT, ER, TPB>, TPB, 0);
        per_sm = b > 0 ? b : 1;
    }
    long long blocks = (io.n + TPB - 1) / TPB;
    if (tune.persistent) blocks = blocks < (long long)per_sm * num_sms ? blocks : (long long)per_sm * num_sms;
    if (blocks < 1) blocks = 1;
    if (blocks > 0x7fffffffLL) blocks = 0x7fffffffLL;
    launch_k(trace_kernel<MODE, COUNT, ER, TPB>, (unsigned)blocks, TPB, 0, st, s, io);
}

template <int MODE, bool COUNT, int ER>
inline void launch_er(const SceneView& s, const TraceIO& io, const TraceTuning& tune, int num_sms, cudaStream_t st) {
    if (COUNT || tune.block == 128) launch_tpb<MODE, COUNT, ER, 128>(s, io, tune, num_sms, st);
    else if (tune.block == 64) launch_tpb<MODE, COUNT, ER, COUNT ? 128 : 64>(s, io, tune, num_sms, st);
    else launch_tpb<MODE, COUNT, ER, COUNT ? 128 : 256>(s, io, tune, num_sms, st);
}

template <int MODE, bool COUNT>
inline void launch_count(const SceneView& s, const TraceIO& io, const TraceTuning& tune, int num_sms,
                         cudaStream_t st) {
    if (tune.empty_run <= 2) launch_er<MODE, COUNT, 2>(s, io, tune, num_sms, st);
    else if (tune.empty_run <= 4) launch_er<MODE, COUNT, 4>(s, io, tune, num_sms, st);
    else if (tune.empty_run <= 8) launch_er<MODE, COUNT, 8>(s, io, tune, num_sms, st);
    else launch_er<MODE, COUNT, 16>(s, io, tune, num_sms, st);
}

template <int MODE, bool COUNT, int G>
inline void launch_wide_g(const SceneView& s, const TraceIO& io, int num_sms, cudaStream_t st) {
    static int per_sm = 0;
    if (per_sm == 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, trace_wide_kernel<MODE, COUNT, G>, 128, 0);
        per_sm = b > 0 ? b : 1;
    }
    launch_k(trace_wide_kernel<MODE, COUNT, G>, (unsigned)(per_sm * num_sms), 128, 0, st, s, io);
}

template <int MODE, bool COUNT>
inline void launch_wide(const SceneView& s, const TraceIO& io, const TraceTuning& tune, int num_sms,
                        cudaStream_t st) {
    if (tune.heavy_lanes <= 4) launch_wide_g<MODE, COUNT, 4>(s, io, num_sms, st);
    else if (tune.heavy_lanes <= 8) launch_wide_g<MODE, COUNT, 8>(s, io, num_sms, st);
    else if (tune.heavy_lanes <= 16) launch_wide_g<MODE, COUNT, 16>(s, io, num_sms, st);
    else launch_wide_g<MODE, COUNT, 32>(s, io, num_sms, st);
}

// As many blocks as fit on the GPU claim the queued rays: each ray's lists
// are long latency chains, so the pass runs as many rays side by side as it
// can hold.
template <int MODE, bool COUNT>
inline void launch_huge(const SceneView& s, const TraceIO& io, int num_sms, cudaStream_t st) {
    static int per_sm = 0;
    if (per_sm == 0) {
        // the staging ring is dynamic shared memory (above the 48 KB of a
        // static allocation for deep rings)
        cudaFuncSetAttribute(trace_huge_kernel<MODE, COUNT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kStageBytes);
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, trace_huge_kernel<MODE, COUNT>, kHugeThreads, kStageBytes);
        per_sm = b > 0 ? b : 1;
    }
    launch_k(trace_huge_kernel<MODE, COUNT>, (unsigned)(per_sm * num_sms), kHugeThreads, kStageBytes, st, s, io);
}

template <int MODE>
inline void launch_mode(const SceneView& s, TraceIO io, const TraceSlot& slot, const TraceTuning& tune, int num_sms,
                        cudaStream_t st) {
    const bool defer = tune.heavy_cell > 0 && slot.defer && slot.defer_cap > 0;
    io.counter = slot.ctr;
    io.defer = defer ? slot.defer : nullptr;
    io.defer_cap = defer ? slot.defer_cap : 0;
    io.heavy = defer ? tune.heavy_cell : kNoHeavy;
    io.refill = refill_for(tune, MODE == MODE_CAMERA || MODE == MODE_FRAME);
    io.huge = defer ? slot.huge : nullptr;
    io.huge_cap = io.huge ? slot.huge_cap : 0;
    cudaMemsetAsync(slot.ctr, 0, 8 * sizeof(unsigned long long), st);
    if (tune.lanes > 1 && !io.ctr) {
        // every ray walked by a group of lanes from its start (the group
        // pass with no queue); lists above kHugeList are still handed to
        // the block-per-ray pass
        io.defer = nullptr;
        io.defer_cap = 0;
        io.heavy = kNoHeavy;
        io.huge = slot.huge;
        io.huge_cap = io.huge ? slot.huge_cap : 0;
        count_launches(io.huge ? 2 : 1);
        if (tune.lanes == 2) launch_wide_g<MODE, false, 2>(s, io, num_sms, st);
        else launch_wide_g<MODE, false, 4>(s, io, num_sms, st);
        if (io.huge) launch_huge<MODE, false>(s, io, num_sms, st);
        return;
    }
    count_launches(defer ? (io.huge ? 3 : 2) : 1);
    if (io.ctr) launch_count<MODE, true>(s, io, tune, num_sms, st);
    else launch_count<MODE, false>(s, io, tune, num_sms, st);
    if (defer) {
        if (io.ctr) launch_wide<MODE, true>(s, io, tune, num_sms, st);
        else launch_wide<MODE, false>(s, io, tune, num_sms, st);
    }
    if (io.huge) {
        if (io.ctr) launch_huge<MODE, true>(s, io, num_sms, st);
        else launch_huge<MODE, false>(s, io, num_sms, st);
    }
}

}  // namespace gridrt
