// shade.cu -- shading wavefront over the tracer (rtg_render).
//
// Restates the reference's per-pixel recursion as levels of rays:
//   Context::traceNearest + IMaterial::shade / IEnvironment::shade
//   Sample::computeShadingNormal / computeHitPosition / computeSpecularVector /
//     computeShadingColor, initLightRay / initShadowRay / initReflectionRay /
//     initRefractionRay (src/rtcore/Sample.cpp)
//   HeadlightMaterial(Color)::shade, PhongMaterial(Color)::shade,
//   SimplePointLight::illuminate, SimpleEnvironment::shade (src/rtplugins/)
// A level is: closest hit of its rays (the tracer's kernels), shadow rays of
// its Phong hits (one per point light) traced any-hit, then a shading pass
// that computes each path's local colour and appends its reflected /
// refracted rays to the next level.  Colours are combined from the deepest
// level up in the reference's order: local, + reflected x reflexion,
// + refracted x (1 - opacity).  vr::vec3f (vrbase) is not in the reference
// checkout: a vector is normalised as v * (1 / sqrt(v.v)), dot products add
// x, y, z left to right, one rounding per operation.
#include <string>
#include <vector>

#include "scene.h"

using namespace gridrt;

namespace {

struct V3 {
    float x, y, z;
};

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 vadd(V3 a, V3 b) { return v3(fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z)); }
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return v3(fsub(a.x, b.x), fsub(a.y, b.y), fsub(a.z, b.z)); }
__device__ __forceinline__ V3 vscale(V3 a, float s) { return v3(fmul(a.x, s), fmul(a.y, s), fmul(a.z, s)); }
__device__ __forceinline__ V3 vmulv(V3 a, V3 b) { return v3(fmul(a.x, b.x), fmul(a.y, b.y), fmul(a.z, b.z)); }
__device__ __forceinline__ float vdot(V3 a, V3 b) { return fadd(fadd(fmul(a.x, b.x), fmul(a.y, b.y)), fmul(a.z, b.z)); }
__device__ __forceinline__ V3 vnorm(V3 a) {
    const float inv = __fdiv_rn(1.0f, __fsqrt_rn(vdot(a, a)));
    return vscale(a, inv);
}
__device__ __forceinline__ V3 vload(const float* p) { return v3(p[0], p[1], p[2]); }
__device__ __forceinline__ V3 vload3(const float (&p)[3]) { return v3(p[0], p[1], p[2]); }
// Sample::reflectDirectionVector: i - n * ((i . n) * 2)
__device__ __forceinline__ V3 vreflect(V3 i, V3 n) { return vsub(i, vscale(n, fmul(vdot(i, n), 2.0f))); }

struct PathRec {
    int32_t child[2];   // reflected, refracted path in the next level (-1: none)
    float coef[2];      // reflexion, 1 - opacity
    float local[3];
    float color[3];
    int32_t pixel;      // level 0: the pixel; deeper: unused
};

struct ShadeArgs {
    const int32_t* idx;          // scene triangles (3 vertex ids each)
    const float* normals;        // per vertex
    const float* colors;         // per vertex or null (white)
    const int32_t* material;     // per triangle or null (0)
    const rtg_material* mats;
    int nmats;
    const rtg_point_light* lights;
    int nlights;
    float bg[3];
    int max_depth;
    float medium;
};

__global__ void raygen_kernel(CameraArgs cam, float4* rays, PathRec* paths, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t px = (int32_t)(i % cam.width), py = (int32_t)(i / cam.width);
        const float us = fmul(fadd(__int2float_rn(px), 0.5f), cam.inv_w);
        const float vs = fmul(fadd(__int2float_rn(py), 0.5f), cam.inv_h);
        float d[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) d[a] = fadd(fadd(cam.base[a], fmul(cam.nu[a], us)), fmul(cam.nv[a], vs));
        rays[2 * i] = make_float4(cam.eye[0], cam.eye[1], cam.eye[2], kRayEpsilon);
        rays[2 * i + 1] = make_float4(d[0], d[1], d[2], kFltMax);
        paths[i].pixel = (int32_t)i;
    }
}

struct HitFrame {
    V3 o, d, n, p;      // ray origin, direction, shading normal, hit position
    float b[3];         // barycentrics of v0, v1, v2
    int32_t tri;
};

__device__ __forceinline__ HitFrame hit_frame(const ShadeArgs& A, const float4* rays, const int4* hits, int64_t j) {
    HitFrame F;
    const float4 ra = rays[2 * j], rb = rays[2 * j + 1];
    const int4 h = hits[j];
    F.o = v3(ra.x, ra.y, ra.z);
    F.d = v3(rb.x, rb.y, rb.z);
    F.tri = h.x;
    const float t = __int_as_float(h.y), u = __int_as_float(h.z), v = __int_as_float(h.w);
    // Hit::v0Coord = 1 - lambda - mue, v1Coord = lambda, v2Coord = mue
    F.b[0] = fsub(fsub(1.0f, u), v);
    F.b[1] = u;
    F.b[2] = v;
    V3 n = v3(0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 3; ++k) n = vadd(n, vscale(vload(A.normals + 3 * (int64_t)A.idx[3 * (int64_t)F.tri + k]), F.b[k]));
    F.n = vnorm(n);
    F.p = vadd(F.o, vscale(F.d, t));
    return F;
}

// Shadow rays of the level's Phong hits: lit[j * nl + i] = 0 no light, 1 lit
// without a test (no shadows cast), 2 lit unless the shadow ray is occluded.
__global__ void shadow_rays_kernel(ShadeArgs A, const float4* rays, const int4* hits, int64_t n, float4* srays,
                                   uint8_t* lit, unsigned long long* nshadow) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const int nl = A.nlights;
        bool phong = false;
        HitFrame F;
        if (hits[j].x >= 0) {
            F = hit_frame(A, rays, hits, j);
            const int m = A.material ? A.material[F.tri] : 0;
            const int type = (m >= 0 && m < A.nmats) ? A.mats[m].type : RTG_MAT_HEADLIGHT;
            phong = type == RTG_MAT_PHONG || type == RTG_MAT_PHONG_COLOR;
        }
        unsigned cnt = 0;
        for (int i = 0; i < nl; ++i) {
            const int64_t s = j * nl + i;
            float4 a = make_float4(0.f, 0.f, 0.f, kRayEpsilon), b = make_float4(0.f, 0.f, 0.f, -1.0f);
            uint8_t l = 0;
            if (phong) {
                // Sample::initLightRay: hit position pushed along the normal by the ray epsilon
                const V3 hp = vadd(F.p, vscale(F.n, kRayEpsilon));
                // SimplePointLight::illuminate: front face, then initShadowRay's n . L > 0
                if (vdot(F.n, F.d) <= 0.0f) {
                    const V3 L = vsub(vload3(A.lights[i].position), hp);
                    if (vdot(F.n, L) > 0.0f) {
                        if (A.lights[i].cast_shadows) {
                            a = make_float4(hp.x, hp.y, hp.z, kRayEpsilon);
                            b = make_float4(L.x, L.y, L.z, 1.0f);
                            l = 2;
                            ++cnt;
                        } else {
                            l = 1;
                        }
                    }
                }
            }
            srays[2 * s] = a;
            srays[2 * s + 1] = b;
            lit[s] = l;
        }
        if (cnt) atomicAdd(nshadow, (unsigned long long)cnt);
    }
}

// Local colour of every path of the level, and its reflected / refracted
// rays appended to the next level (when depth < max_depth).
__global__ void shade_kernel(ShadeArgs A, const float4* rays, const int4* hits, int64_t n, const uint8_t* lit,
                             const uint8_t* occ, int depth, PathRec* paths, float4* next_rays,
                             unsigned long long* next_count) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        PathRec& P = paths[j];
        P.child[0] = P.child[1] = -1;
        P.coef[0] = P.coef[1] = 0.0f;
        if (hits[j].x < 0) {   // SimpleEnvironment::shade
            P.local[0] = A.bg[0];
            P.local[1] = A.bg[1];
            P.local[2] = A.bg[2];
            continue;
        }
        HitFrame F = hit_frame(A, rays, hits, j);
        const int m = A.material ? A.material[F.tri] : 0;
        rtg_material M;
        if (m >= 0 && m < A.nmats) {
            M = A.mats[m];
        } else {
            M.type = RTG_MAT_HEADLIGHT;
            M.ambient[0] = M.ambient[1] = M.ambient[2] = 0.1f;
        }
        V3 vcol = v3(1.f, 1.f, 1.f);
        if (A.colors && (M.type == RTG_MAT_HEADLIGHT || M.type == RTG_MAT_PHONG)) {
            vcol = v3(0.f, 0.f, 0.f);
#pragma unroll
            for (int k = 0; k < 3; ++k)
                vcol = vadd(vcol, vscale(vload(A.colors + 3 * (int64_t)A.idx[3 * (int64_t)F.tri + k]), F.b[k]));
        }
        const V3 amb = vload3(M.ambient);
        V3 out;
        if (M.type == RTG_MAT_HEADLIGHT || M.type == RTG_MAT_HEADLIGHT_COLOR) {
            // (ambient + (c - ambient) * nDotD) * c, d normalised
            const V3 c = M.type == RTG_MAT_HEADLIGHT ? vcol : vload3(M.diffuse);
            const float ndd = -vdot(F.n, vnorm(F.d));
            out = vmulv(vadd(amb, vscale(vsub(c, amb), ndd)), c);
        } else {
            const V3 spec = vnorm(vreflect(F.d, F.n));
            const V3 hp = vadd(F.p, vscale(F.n, kRayEpsilon));
            V3 dif = v3(0.f, 0.f, 0.f), spc = v3(0.f, 0.f, 0.f);
            for (int i = 0; i < A.nlights; ++i) {
                const int64_t s = j * A.nlights + i;
                const uint8_t l = lit[s];
                if (l == 0 || (l == 2 && occ[s] != 0)) continue;
                const V3 Ld = vnorm(vsub(vload3(A.lights[i].position), hp));
                const V3 lc = vload3(A.lights[i].intensity);
                dif = vadd(dif, vscale(lc, vdot(F.n, Ld)));
                if (M.type == RTG_MAT_PHONG || M.specular_exponent > 0.0f) {
                    const float sdl = vdot(spec, Ld);
                    if (sdl > 0.0f) spc = vadd(spc, vscale(lc, powf(sdl, M.specular_exponent)));
                }
            }
            const V3 sc = vload3(M.specular);
            if (M.type == RTG_MAT_PHONG) {
                out = vadd(vmulv(vcol, vadd(amb, dif)), vmulv(sc, spc));
            } else {
                out = vmulv(vload3(M.diffuse), dif);
                out = vadd(out, vadd(amb, vmulv(sc, spc)));
            }
            if (depth < A.max_depth) {
                if (M.reflexion > 0.0f) {
                    const V3 r = vreflect(F.d, F.n);
                    const unsigned long long c = atomicAdd(next_count, 1ull);
                    next_rays[2 * c] = make_float4(F.p.x, F.p.y, F.p.z, kRayEpsilon);
                    next_rays[2 * c + 1] = make_float4(r.x, r.y, r.z, kFltMax);
                    P.child[0] = (int32_t)c;
                    P.coef[0] = M.reflexion;
                }
                if (M.opacity < 1.0f) {
                    const bool front = vdot(F.n, F.d) <= 0.0f;
                    const V3 nn = front ? F.n : vscale(F.n, -1.0f);
                    const float ratio = front ? __fdiv_rn(A.medium, M.refraction_index)
                                              : __fdiv_rn(M.refraction_index, A.medium);
                    const V3 nd = vnorm(F.d);
                    const float cosI = -vdot(nn, nd);
                    const float cosT2 = fsub(1.0f, fmul(fmul(ratio, ratio), fsub(1.0f, fmul(cosI, cosI))));
                    if (cosT2 > 0.0f) {
                        const float cosT = __fsqrt_rn(cosT2);
                        const V3 t = vadd(vscale(nd, ratio), vscale(nn, fsub(fmul(ratio, cosI), cosT)));
                        const unsigned long long c = atomicAdd(next_count, 1ull);
                        next_rays[2 * c] = make_float4(F.p.x, F.p.y, F.p.z, kRayEpsilon);
                        next_rays[2 * c + 1] = make_float4(t.x, t.y, t.z, kFltMax);
                        P.child[1] = (int32_t)c;
                        P.coef[1] = fsub(1.0f, M.opacity);
                    }
                }
            }
        }
        P.local[0] = out.x;
        P.local[1] = out.y;
        P.local[2] = out.z;
    }
}

// Colours bottom-up: local, + reflected x reflexion, + refracted x (1 - opacity).
__global__ void combine_kernel(PathRec* paths, int64_t n, const PathRec* next) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        PathRec& P = paths[j];
        float c[3] = {P.local[0], P.local[1], P.local[2]};
        for (int k = 0; k < 2; ++k) {
            if (P.child[k] < 0) continue;
            const PathRec& C = next[P.child[k]];
            for (int a = 0; a < 3; ++a) c[a] = fadd(c[a], fmul(C.color[a], P.coef[k]));
        }
        P.color[0] = c[0];
        P.color[1] = c[1];
        P.color[2] = c[2];
    }
}

__global__ void write_rgb_kernel(const PathRec* paths, int64_t n, float* rgb) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = paths[j].pixel;
        rgb[3 * p] = paths[j].color[0];
        rgb[3 * p + 1] = paths[j].color[1];
        rgb[3 * p + 2] = paths[j].color[2];
    }
}

int grid_for(int64_t n, int sms) {
    int64_t b = (n + 255) / 256;
    const int64_t cap = 16LL * (sms > 0 ? sms : 1);
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

struct Level {
    int64_t n = 0;
    float4* rays = nullptr;
    int4* hits = nullptr;
    PathRec* paths = nullptr;
};

rtg_status sfail(rtg_status s, const std::string& msg) {
    set_last_error(msg);
    return s;
}

}  // namespace

extern "C" rtg_status rtg_render(rtg_scene s, const rtg_camera* cam, const rtg_shading* sh, float* d_rgb,
                                 int64_t* rays_out, void* stream) {
    if (!s || !cam || !sh || !d_rgb) return sfail(RTG_INVALID_PARAM, "NULL argument");
    if (!s->built) return sfail(RTG_NOT_BUILT, "scene not built");
    if (!camera_ok(cam) || cam->order != RTG_ORDER_SCANLINE)
        return sfail(RTG_INVALID_PARAM, "render needs a scanline camera of positive size");
    if (!sh->d_normals || sh->nmaterials < 0 || (sh->nmaterials && !sh->materials) || sh->nlights < 0 ||
        (sh->nlights && !sh->lights) || sh->max_depth < 0 || sh->max_depth > 16)
        return sfail(RTG_INVALID_PARAM, "bad shading description");
    if (cudaSetDevice(s->device) != cudaSuccess) return sfail(RTG_DEVICE_ERROR, "cudaSetDevice");
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    const int64_t npix = (int64_t)cam->width * cam->height;
    const int nl = sh->nlights;
    std::vector<void*> owned;
    rtg_status rc = RTG_OK;
    auto alloc = [&](void** p, size_t bytes) -> bool {
        *p = nullptr;
        if (cudaMallocAsync(p, bytes ? bytes : 16, st) != cudaSuccess) {
            rc = sfail(RTG_NO_MEMORY, "render buffers");
            return false;
        }
        owned.push_back(*p);
        return true;
    };
    auto cleanup = [&]() {
        for (void* p : owned) cudaFreeAsync(p, st);
        cudaStreamSynchronize(st);
    };
    rtg_material* d_mats = nullptr;
    rtg_point_light* d_lights = nullptr;
    unsigned long long* d_cnt = nullptr;   // [0] next level, [1] shadow rays
    if (!alloc((void**)&d_mats, sizeof(rtg_material) * (size_t)sh->nmaterials) ||
        !alloc((void**)&d_lights, sizeof(rtg_point_light) * (size_t)nl) ||
        !alloc((void**)&d_cnt, 2 * sizeof(unsigned long long))) {
        cleanup();
        return rc;
    }
    if (sh->nmaterials)
        cudaMemcpyAsync(d_mats, sh->materials, sizeof(rtg_material) * sh->nmaterials, cudaMemcpyHostToDevice, st);
    if (nl) cudaMemcpyAsync(d_lights, sh->lights, sizeof(rtg_point_light) * nl, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(d_cnt, 0, 2 * sizeof(unsigned long long), st);

    ShadeArgs A;
    A.idx = s->d_idx;
    A.normals = sh->d_normals;
    A.colors = sh->d_colors;
    A.material = sh->d_material;
    A.mats = d_mats;
    A.nmats = sh->nmaterials;
    A.lights = d_lights;
    A.nlights = nl;
    for (int a = 0; a < 3; ++a) A.bg[a] = sh->background[a];
    A.max_depth = sh->max_depth;
    A.medium = sh->medium_index;

    std::vector<Level> levels(1);
    levels[0].n = npix;
    if (!alloc((void**)&levels[0].rays, 32 * (size_t)npix) || !alloc((void**)&levels[0].hits, 16 * (size_t)npix) ||
        !alloc((void**)&levels[0].paths, sizeof(PathRec) * (size_t)npix)) {
        cleanup();
        return rc;
    }
    const int sms = s->num_sms;
    count_launches(1);
    raygen_kernel<<<grid_for(npix, sms), 256, 0, st>>>(camera_args(cam), levels[0].rays, levels[0].paths, npix);
    int64_t traced = 0;
    for (int depth = 0;; ++depth) {
        Level& L = levels[depth];
        const SceneView v = scene_view(s);
        launch_trace_nearest(v, L.rays, L.n, L.hits, nullptr, scene_counter(s), s->tune, sms, st);
        traced += L.n;
        float4* srays = nullptr;
        uint8_t* lit = nullptr;
        uint8_t* occ = nullptr;
        if (nl) {
            const size_t ns = (size_t)L.n * nl;
            if (!alloc((void**)&srays, 32 * ns) || !alloc((void**)&lit, ns) || !alloc((void**)&occ, ns)) break;
            count_launches(1);
            shadow_rays_kernel<<<grid_for(L.n, sms), 256, 0, st>>>(A, L.rays, L.hits, L.n, srays, lit, d_cnt + 1);
            launch_trace_any(v, srays, (int64_t)ns, occ, nullptr, scene_counter(s), s->tune, sms, st);
        }
        Level next;
        const bool more = depth < sh->max_depth;
        if (more) {
            next.n = 2 * L.n;
            if (!alloc((void**)&next.rays, 32 * (size_t)next.n)) break;
        }
        cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long), st);
        count_launches(1);
        shade_kernel<<<grid_for(L.n, sms), 256, 0, st>>>(A, L.rays, L.hits, L.n, lit, occ, depth, L.paths, next.rays,
                                                          d_cnt);
        if (!more) break;
        unsigned long long cnt = 0;
        if (cudaMemcpyAsync(&cnt, d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            rc = sfail(RTG_DEVICE_ERROR, "render level count");
            break;
        }
        if (cnt == 0) break;
        next.n = (int64_t)cnt;
        if (!alloc((void**)&next.hits, 16 * (size_t)next.n) || !alloc((void**)&next.paths, sizeof(PathRec) * next.n))
            break;
        levels.push_back(next);
    }
    if (rc == RTG_OK) {
        for (int d = (int)levels.size() - 1; d >= 0; --d) {
            count_launches(1);
            combine_kernel<<<grid_for(levels[d].n, sms), 256, 0, st>>>(
                levels[d].paths, levels[d].n, d + 1 < (int)levels.size() ? levels[d + 1].paths : nullptr);
        }
        count_launches(1);
        write_rgb_kernel<<<grid_for(npix, sms), 256, 0, st>>>(levels[0].paths, npix, d_rgb);
        unsigned long long nsh = 0;
        cudaMemcpyAsync(&nsh, d_cnt + 1, sizeof(nsh), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess)
            rc = sfail(RTG_DEVICE_ERROR, "render kernels");
        if (rays_out) *rays_out = traced + (int64_t)nsh;
    }
    cleanup();
    return rc;
}
