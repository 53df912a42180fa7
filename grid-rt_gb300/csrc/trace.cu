// trace.cu -- one-ray-per-thread 3D-DDA traversal with Moller-Trumbore.
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
// triangles are the reference's.  Only the triangle test differs (MT instead
// of Wald's projection test), which moves t / u / v by a few ulps and can flip
// the winner between triangles whose t differ by less than that (near-ties).
#include "common.cuh"
#include "kernels.h"

namespace gridrt {

static constexpr unsigned FULL = 0xffffffffu;

static unsigned long long g_launches = 0;
void count_launches(int n) { __atomic_add_fetch(&g_launches, (unsigned long long)n, __ATOMIC_RELAXED); }
unsigned long long launches_so_far() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

struct PLite {
    float bmin[3], bmax[3], cell[3], inv[3];
    int32_t res[3];
    int32_t pad;
};

__device__ __forceinline__ void load_params(const GridParams* __restrict__ gp, PLite& P) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        P.bmin[d] = gp->bmin[d];
        P.bmax[d] = gp->bmax[d];
        P.cell[d] = gp->cell[d];
        P.inv[d] = gp->inv[d];
        P.res[d] = gp->res[d];
    }
}

struct TraceResult {
    int32_t id;
    float t, u, v;
    uint32_t cells, tests;
};

// Reported hit values of the winning triangle.  Moller-Trumbore's u, v and t
// come from dot products of the (large) origin-to-vertex vector, which cancel
// badly for small triangles seen from far away; the winner's t is therefore
// re-derived from the plane equation t = ((v0 - o).n) / (d.n) and u, v from
// the hit point P = o + t*d projected on the triangle's dominant plane (the
// quantities Wald's test evaluates, src/rtcore/RayTriIntersection.cpp:15-47).
// The accept / reject decisions above stay Moller-Trumbore's.
__device__ __forceinline__ void refine_hit(const float4* __restrict__ tris, TraceResult& R, const float o[3],
                                           const float d[3]) {
    const float4 A = __ldg(tris + 3 * (int64_t)R.id);
    const float4 B = __ldg(tris + 3 * (int64_t)R.id + 1);
    const float4 C = __ldg(tris + 3 * (int64_t)R.id + 2);
    const float nx = B.y * C.z - B.z * C.y, ny = B.z * C.x - B.x * C.z, nz = B.x * C.y - B.y * C.x;
    const float num = (A.x - o[0]) * nx + (A.y - o[1]) * ny + (A.z - o[2]) * nz;
    const float den = d[0] * nx + d[1] * ny + d[2] * nz;
    const float t = num / den;
    const float wx = (o[0] + t * d[0]) - A.x, wy = (o[1] + t * d[1]) - A.y, wz = (o[2] + t * d[2]) - A.z;
    const float ax = fabsf(nx), ay = fabsf(ny), az = fabsf(nz);
    float e1a, e1b, e2a, e2b, wa, wb;
    if (ax > ay && ax > az) {          // drop x
        e1a = B.y; e1b = B.z; e2a = C.y; e2b = C.z; wa = wy; wb = wz;
    } else if (ay > az) {              // drop y
        e1a = B.z; e1b = B.x; e2a = C.z; e2b = C.x; wa = wz; wb = wx;
    } else {                           // drop z
        e1a = B.x; e1b = B.y; e2a = C.x; e2b = C.y; wa = wx; wb = wy;
    }
    const float D = e1a * e2b - e2a * e1b;
    const float u = (wa * e2b - e2a * wb) / D;
    const float v = (e1a * wb - wa * e1b) / D;
    if (isfinite(t) && isfinite(u) && isfinite(v)) {
        R.t = t;
        R.u = u;
        R.v = v;
    }
}

// ANY = false: closest hit.  ANY = true: returns id >= 0 iff occluded before tmax.
template <bool ANY>
__device__ __forceinline__ TraceResult traverse(const PLite& P, const int32_t* __restrict__ offsets,
                                                const int32_t* __restrict__ ids, const float4* __restrict__ tris,
                                                const float o[3], const float d[3], float tnear, float tfar) {
    TraceResult R;
    R.id = -1; R.t = 0.f; R.u = 0.f; R.v = 0.f; R.cells = 0; R.tests = 0;
    const float tmax = tfar;
    // Ray::update (include/rt/Ray.h:26-37)
    float inv[3];
    int32_t sgn[3], sbit[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        inv[a] = frcp(d[a]);
        sgn[a] = d[a] < 0.0f ? -1 : (d[a] > 0.0f ? 1 : 0);
        sbit[a] = (__float_as_uint(d[a]) >> 31);
    }
    // AabbIntersection::clipRay (src/rtcore/AabbIntersection.cpp:37-63)
    float rn = tnear, rf = tfar;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float tn = fmul(fsub(P.bmin[a], o[a]), inv[a]);
        const float tf = fmul(fsub(P.bmax[a], o[a]), inv[a]);
        rn = vmax(rn, vmin(tn, tf));
        rf = vmin(rf, vmax(tn, tf));
    }
    if (rn > rf) return R;
    tnear = rn;
    // traverse3ddda setup (src/rtplugins/UniformGridAccStruct.cpp:122-149)
    const int32_t nx = P.res[0], ny = P.res[1], nz = P.res[2];
    int32_t c3[3];
    float tMax[3], tDelta[3];
    int32_t out[3];
    const int32_t nn[3] = {nx, ny, nz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float sp = fadd(o[a], fmul(d[a], tnear));
        c3[a] = vclamp(world_to_voxel(sp, P.bmin[a], P.inv[a]), 0, nn[a] - 1);
        out[a] = -sbit[a] + nn[a] * (sbit[a] ^ 1);
        tDelta[a] = vabs(fmul(P.cell[a], inv[a]));
        tMax[a] = fmul(fsub(voxel_to_world(c3[a] + (sbit[a] ^ 1), P.cell[a], P.bmin[a]), o[a]), inv[a]);
    }
    int32_t x = c3[0], y = c3[1], z = c3[2];
    float tMaxX = tMax[0], tMaxY = tMax[1], tMaxZ = tMax[2];
    const float lo = fsub(tnear, kHitEpsilon);
    const int32_t nxy = nx * ny;
    // A DDA walk visits at most nx+ny+nz-2 cells; the bound only guards
    // against non-finite rays (a zero direction component) looping forever.
    int32_t budget = nx + ny + nz + 3;
    float best = kFltMax;
    do {
        const int32_t c = x + y * nx + z * nxy;
        const int32_t b = __ldg(offsets + c), e = __ldg(offsets + c + 1);
        ++R.cells;
        if (b != e) {
            const float cell_exit = vmin(vmin(tMaxX, tMaxY), tMaxZ);
            const float hi = fadd(cell_exit, kHitEpsilon);
            R.tests += (uint32_t)(e - b);
            for (int32_t i = b; i < e; ++i) {
                const int32_t tid = __ldg(ids + i);
                const float4 A = __ldg(tris + 3 * (int64_t)tid);
                const float4 B = __ldg(tris + 3 * (int64_t)tid + 1);
                const float4 C = __ldg(tris + 3 * (int64_t)tid + 2);
                // Moller-Trumbore: v0 = A.xyz, e1 = B.xyz, e2 = C.xyz
                const float tvx = o[0] - A.x, tvy = o[1] - A.y, tvz = o[2] - A.z;
                const float px = d[1] * C.z - d[2] * C.y;
                const float py = d[2] * C.x - d[0] * C.z;
                const float pz = d[0] * C.y - d[1] * C.x;
                const float det = B.x * px + B.y * py + B.z * pz;
                const float idet = frcp(det);
                const float u = (tvx * px + tvy * py + tvz * pz) * idet;
                const float qx = tvy * B.z - tvz * B.y;
                const float qy = tvz * B.x - tvx * B.z;
                const float qz = tvx * B.y - tvy * B.x;
                const float v = (d[0] * qx + d[1] * qy + d[2] * qz) * idet;
                const float t = (C.x * qx + C.y * qy + C.z * qz) * idet;
                const bool acc = (t < best) && (t >= lo) && (t <= hi) && (u >= 0.0f) && (v >= 0.0f) &&
                                 ((1.0f - u) - v >= 0.0f);
                if (acc) {
                    if (ANY && t < tmax) {
                        R.id = tid; R.t = t; R.u = u; R.v = v;
                        return R;
                    }
                    best = t;
                    R.id = tid; R.t = t; R.u = u; R.v = v;
                }
            }
            if (best < kFltMax) {
                if (ANY) {
                    R.id = -1;   // first cell with a hit decides: not before tmax
                } else {
                    refine_hit(tris, R, o, d);
                }
                return R;
            }
        }
        if (tMaxX < tMaxY && tMaxX < tMaxZ) {
            x += sgn[0];
            tMaxX = fadd(tMaxX, tDelta[0]);
        } else if (tMaxY < tMaxZ) {
            y += sgn[1];
            tMaxY = fadd(tMaxY, tDelta[1]);
        } else {
            z += sgn[2];
            tMaxZ = fadd(tMaxZ, tDelta[2]);
        }
    } while (x != out[0] && y != out[1] && z != out[2] && --budget > 0);
    R.id = -1;
    return R;
}

template <bool COUNT>
__device__ __forceinline__ void add_counters(TraceCounters* ctr, uint32_t cells, uint32_t tests, bool valid) {
    if (!COUNT) return;
    unsigned long long r = valid ? 1 : 0, c = cells, t = tests;
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

template <bool COUNT>
__global__ void __launch_bounds__(256) trace_nearest_kernel(SceneView s, const float4* __restrict__ rays, int64_t n,
                                                            int4* __restrict__ hits, TraceCounters* ctr) {
    PLite P;
    load_params(s.params, P);
    const bool failed = build_failed(s.params->status);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        TraceResult R;
        R.cells = R.tests = 0;
        if (i < n) {
            const float4 a = __ldg(rays + 2 * i), b = __ldg(rays + 2 * i + 1);
            const float o[3] = {a.x, a.y, a.z}, d[3] = {b.x, b.y, b.z};
            if (!failed) R = traverse<false>(P, s.offsets, s.ids, s.tris, o, d, a.w, b.w);
            else R.id = -1;
            hits[i] = make_int4(R.id, __float_as_int(R.t), __float_as_int(R.u), __float_as_int(R.v));
        }
        add_counters<COUNT>(ctr, R.cells, R.tests, i < n);
    }
}

template <bool COUNT>
__global__ void __launch_bounds__(256) trace_any_kernel(SceneView s, const float4* __restrict__ rays, int64_t n,
                                                        uint8_t* __restrict__ occ, TraceCounters* ctr) {
    PLite P;
    load_params(s.params, P);
    const bool failed = build_failed(s.params->status);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        TraceResult R;
        R.cells = R.tests = 0;
        bool valid = false;
        if (i < n) {
            const float4 a = __ldg(rays + 2 * i), b = __ldg(rays + 2 * i + 1);
            uint8_t r = 2;   // no shadow ray (tmax < 0)
            if (b.w >= 0.0f) {
                const float o[3] = {a.x, a.y, a.z}, d[3] = {b.x, b.y, b.z};
                if (!failed) R = traverse<true>(P, s.offsets, s.ids, s.tris, o, d, a.w, b.w);
                else R.id = -1;
                r = R.id >= 0 ? 1 : 0;
                valid = true;
            }
            occ[i] = r;
        }
        add_counters<COUNT>(ctr, R.cells, R.tests, valid);
    }
}

__device__ __forceinline__ void ray_pixel(int64_t i, const CameraArgs& cam, int32_t& px, int32_t& py) {
    if (cam.order == 1) {
        const int64_t tile = i >> 6;
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

// Primary rays at pixel centres (PinholeCamera::getRayDirection,
// src/rtplugins/PinholeCamera.cpp:131-137), then optionally the shadow ray of
// SimplePointLight::illuminate (src/rtplugins/SimplePointLight.cpp:18-52).
template <bool COUNT>
__global__ void __launch_bounds__(256) trace_camera_kernel(SceneView s, CameraArgs cam, int4* __restrict__ hits,
                                                           float3 light, int has_light,
                                                           float4* __restrict__ shadow_rays, TraceCounters* ctr) {
    PLite P;
    load_params(s.params, P);
    const bool failed = build_failed(s.params->status);
    const int64_t n = (int64_t)cam.width * cam.height;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        TraceResult R;
        R.cells = R.tests = 0;
        if (i < n) {
            int32_t px, py;
            ray_pixel(i, cam, px, py);
            const float us = fmul(fadd(__int2float_rn(px), 0.5f), cam.inv_w);
            const float vs = fmul(fadd(__int2float_rn(py), 0.5f), cam.inv_h);
            float d[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) d[a] = fadd(fadd(cam.base[a], fmul(cam.nu[a], us)), fmul(cam.nv[a], vs));
            const float o[3] = {cam.eye[0], cam.eye[1], cam.eye[2]};
            if (!failed) R = traverse<false>(P, s.offsets, s.ids, s.tris, o, d, kRayEpsilon, kFltMax);
            else R.id = -1;
            hits[i] = make_int4(R.id, __float_as_int(R.t), __float_as_int(R.u), __float_as_int(R.v));
            if (shadow_rays) {
                float4 sa = make_float4(0.f, 0.f, 0.f, kRayEpsilon), sb = make_float4(0.f, 0.f, 0.f, -1.0f);
                if (R.id >= 0 && has_light) {
                    // Sample::computeHitPosition, flat normal facing the ray,
                    // initLightRay offset and initShadowRay (src/rtcore/Sample.cpp:22-42,177-180,224-236)
                    const float4 B = __ldg(s.tris + 3 * (int64_t)R.id + 1);
                    const float4 C = __ldg(s.tris + 3 * (int64_t)R.id + 2);
                    float nx = B.y * C.z - B.z * C.y, ny = B.z * C.x - B.x * C.z, nz = B.x * C.y - B.y * C.x;
                    const float rl = rsqrtf(nx * nx + ny * ny + nz * nz);
                    nx *= rl; ny *= rl; nz *= rl;
                    if (nx * d[0] + ny * d[1] + nz * d[2] > 0.0f) { nx = -nx; ny = -ny; nz = -nz; }
                    const float hx = o[0] + d[0] * R.t + nx * kRayEpsilon;
                    const float hy = o[1] + d[1] * R.t + ny * kRayEpsilon;
                    const float hz = o[2] + d[2] * R.t + nz * kRayEpsilon;
                    const float lx = light.x - hx, ly = light.y - hy, lz = light.z - hz;
                    if (nx * lx + ny * ly + nz * lz > 0.0f) {
                        sa = make_float4(hx, hy, hz, kRayEpsilon);
                        sb = make_float4(lx, ly, lz, 1.0f);
                    }
                }
                shadow_rays[2 * i] = sa;
                shadow_rays[2 * i + 1] = sb;
            }
        }
        add_counters<COUNT>(ctr, R.cells, R.tests, i < n);
    }
}

__global__ void deform_kernel(const float* __restrict__ base, const float* __restrict__ nrm, float* __restrict__ out,
                              int64_t nverts, float amp, float freq, float phase) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nverts; i += stride) {
        const float px = base[3 * i], py = base[3 * i + 1], pz = base[3 * i + 2];
        const float s = amp * sinf(freq * px + phase);
        out[3 * i] = px + s * nrm[3 * i];
        out[3 * i + 1] = py + s * nrm[3 * i + 1];
        out[3 * i + 2] = pz + s * nrm[3 * i + 2];
    }
}

static int grid_for(int64_t n, int num_sms) {
    int64_t blocks = (n + 255) / 256;
    const int64_t cap = (int64_t)num_sms * 64;
    if (blocks > cap) blocks = cap;
    return (int)(blocks < 1 ? 1 : blocks);
}

void launch_trace_nearest(const SceneView& s, const float4* rays, int64_t n, int4* hits, TraceCounters* ctr,
                          int num_sms, cudaStream_t st) {
    if (n <= 0) return;
    count_launches(1);
    if (ctr) trace_nearest_kernel<true><<<grid_for(n, num_sms), 256, 0, st>>>(s, rays, n, hits, ctr);
    else trace_nearest_kernel<false><<<grid_for(n, num_sms), 256, 0, st>>>(s, rays, n, hits, ctr);
}

void launch_trace_any(const SceneView& s, const float4* rays, int64_t n, uint8_t* occ, TraceCounters* ctr,
                      int num_sms, cudaStream_t st) {
    if (n <= 0) return;
    count_launches(1);
    if (ctr) trace_any_kernel<true><<<grid_for(n, num_sms), 256, 0, st>>>(s, rays, n, occ, ctr);
    else trace_any_kernel<false><<<grid_for(n, num_sms), 256, 0, st>>>(s, rays, n, occ, ctr);
}

void launch_trace_camera(const SceneView& s, const CameraArgs& cam, int4* hits, const float* light,
                         float4* shadow_rays, TraceCounters* ctr, int num_sms, cudaStream_t st) {
    const int64_t n = (int64_t)cam.width * cam.height;
    if (n <= 0) return;
    count_launches(1);
    const float3 L = light ? make_float3(light[0], light[1], light[2]) : make_float3(0.f, 0.f, 0.f);
    if (ctr)
        trace_camera_kernel<true><<<grid_for(n, num_sms), 256, 0, st>>>(s, cam, hits, L, light != nullptr,
                                                                         shadow_rays, ctr);
    else
        trace_camera_kernel<false><<<grid_for(n, num_sms), 256, 0, st>>>(s, cam, hits, L, light != nullptr,
                                                                          shadow_rays, ctr);
}

void launch_deform(const float* base, const float* normals, float* out, int64_t nverts, float amp, float freq,
                   float phase, cudaStream_t st) {
    if (nverts <= 0) return;
    count_launches(1);
    int64_t blocks = (nverts + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    deform_kernel<<<(int)blocks, 256, 0, st>>>(base, normals, out, nverts, amp, freq, phase);
}

}  // namespace gridrt
