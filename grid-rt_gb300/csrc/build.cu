// build.cu -- per-frame uniform-grid construction on the device.
//
// Replaces rtp::UniformGridAccStructBuilder::buildUniformGrid
// (src/rtplugins/UniformGridAccStructBuilder.cpp:71-149) and the GPU grid
// passes the reference drove through GLSL (shaders/countCellFP.glsl:39-73,
// gridAccumVP_sem_GS.glsl:27-38, gridFP.glsl:60-131).  Output is a CSR grid:
// offsets[ncells + 1] and ids[nrefs], each cell's list sorted by triangle id,
// bit-identical to the reference's per-cell std::vector lists.
//
// Pipeline (no host round trip):
//   records       the trace's triangle records: Moller-Trumbore {v0|id, e1,
//                 e2} and the reference's TriAccel record (on a stream of its
//                 own beside the passes below, joined at the end)
//   bbox_params   scene box (exact min/max), 1% enlargement, resolution rule;
//                 the last block derives the grid parameters on the device;
//                 also clears the offsets and the occupancy bitmap
//   zero_offsets  the clear alone (host-resolved parameters)
//   count         warp-cooperative expansion of each triangle's cell range;
//                 warp-aggregated atomicAdd of per-cell counts
//   scan x2       tile sums, then the in-place inclusive scan of the counts
//                 (cursors = cell ends), occupancy bits and the sort queues
//   scatter       same expansion; warp-aggregated atomicSub on the cursors,
//                 which leaves them equal to the exclusive cell starts
//   sort x3       per-cell sort by triangle id: thread network (<= 8), warp
//                 bitonic (<= 256), block bitonic in shared memory (<= 4096),
//                 shared-memory bitmap compaction for larger cells (ids
//                 within a cell are unique)
#include "common.cuh"
#include "kernels.h"

#include <climits>
#include <cooperative_groups.h>

namespace gridrt {

static constexpr unsigned FULL = 0xffffffffu;

// Batch launches use one flat grid: blocks [first[t], first[t+1]) work on
// task t (first[] is a prefix table over the tasks' block counts).
__device__ __forceinline__ int block_task(const int* __restrict__ first, int ntasks) {
    int lo = 0, hi = ntasks - 1;
    const int b = (int)blockIdx.x;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(first + mid) <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// bbox + grid parameters
// ---------------------------------------------------------------------------
// Aabb::buildFrom / expandBy (src/rtcore/Aabb.cpp:11-53): min/max per axis.
// A NaN coordinate never wins a comparison there, so it is skipped here too.
// The same blocks first clear the whole offsets capacity (the count pass
// adds into it) and the occupancy bitmap, which needs no grid parameters.
__device__ __forceinline__ void zero_capacity(int32_t* __restrict__ offsets, uint32_t* __restrict__ occ,
                                              int64_t cell_cap, unsigned vbx, unsigned vgx) {
    const int64_t t0 = (int64_t)vbx * blockDim.x + threadIdx.x, nt = (int64_t)vgx * blockDim.x;
    const int64_t n4 = cell_cap >> 2;
    for (int64_t i = t0; i < n4; i += nt) {
        reinterpret_cast<int4*>(offsets)[i] = make_int4(0, 0, 0, 0);
        if (occ) reinterpret_cast<uint4*>(occ)[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    for (int64_t i = (n4 << 2) + t0; i < cell_cap; i += nt) {
        offsets[i] = 0;
        if (occ) occ[i] = 0u;
    }
}

__device__ __forceinline__ void bbox_params_body(const float* __restrict__ verts, int64_t nverts,
                                                          BuildWork* w, GridParams* p, int32_t k, int64_t ntris,
                                                          int64_t cell_cap, unsigned vbx, unsigned vgx) {
    float mn0 = INFINITY, mn1 = INFINITY, mn2 = INFINITY;
    float mx0 = -INFINITY, mx1 = -INFINITY, mx2 = -INFINITY;
    const int64_t stride = (int64_t)vgx * blockDim.x;
    for (int64_t i = (int64_t)vbx * blockDim.x + threadIdx.x; i < nverts; i += stride) {
        const float a = __ldg(verts + 3 * i), b = __ldg(verts + 3 * i + 1), c = __ldg(verts + 3 * i + 2);
        mn0 = a < mn0 ? a : mn0; mx0 = a > mx0 ? a : mx0;
        mn1 = b < mn1 ? b : mn1; mx1 = b > mx1 ? b : mx1;
        mn2 = c < mn2 ? c : mn2; mx2 = c > mx2 ? c : mx2;
    }
    for (int o = 16; o > 0; o >>= 1) {
        float t;
        t = __shfl_xor_sync(FULL, mn0, o); mn0 = t < mn0 ? t : mn0;
        t = __shfl_xor_sync(FULL, mn1, o); mn1 = t < mn1 ? t : mn1;
        t = __shfl_xor_sync(FULL, mn2, o); mn2 = t < mn2 ? t : mn2;
        t = __shfl_xor_sync(FULL, mx0, o); mx0 = t > mx0 ? t : mx0;
        t = __shfl_xor_sync(FULL, mx1, o); mx1 = t > mx1 ? t : mx1;
        t = __shfl_xor_sync(FULL, mx2, o); mx2 = t > mx2 ? t : mx2;
    }
    __shared__ float red[6][8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        red[0][wid] = mn0; red[1][wid] = mn1; red[2][wid] = mn2;
        red[3][wid] = mx0; red[4][wid] = mx1; red[5][wid] = mx2;
    }
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        for (int i = 1; i < nw; ++i) {
            mn0 = red[0][i] < mn0 ? red[0][i] : mn0;
            mn1 = red[1][i] < mn1 ? red[1][i] : mn1;
            mn2 = red[2][i] < mn2 ? red[2][i] : mn2;
            mx0 = red[3][i] > mx0 ? red[3][i] : mx0;
            mx1 = red[4][i] > mx1 ? red[4][i] : mx1;
            mx2 = red[5][i] > mx2 ? red[5][i] : mx2;
        }
        atomicMin(&w->keys[0], f2key(mn0));
        atomicMin(&w->keys[1], f2key(mn1));
        atomicMin(&w->keys[2], f2key(mn2));
        atomicMax(&w->keys[3], f2key(mx0));
        atomicMax(&w->keys[4], f2key(mx1));
        atomicMax(&w->keys[5], f2key(mx2));
        __threadfence();
        const uint32_t ticket = atomicAdd(&w->ticket, 1u);
        last = (ticket == vgx - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();

    // ---- last block: grid parameters --------------------------------------
    float mn[3], mx[3];
    for (int d = 0; d < 3; ++d) {
        mn[d] = key2f(atomicAdd(&w->keys[d], 0u));
        mx[d] = key2f(atomicAdd(&w->keys[3 + d], 0u));
        w->keys[d] = 0xffffffffu;   // reset for the next build
        w->keys[3 + d] = 0u;
    }
    w->ticket = 0u;
    w->nsort[0] = w->nsort[1] = w->nsort[2] = w->nsort[3] = 0u;
    // Aabb::scaleBy(0.01f) with planar tolerance 0.01f (src/rtcore/Aabb.cpp:78-91)
    for (int d = 0; d < 3; ++d) {
        const float s = (mn[d] == mx[d]) ? 0.01f : fmul(vabs(fsub(mx[d], mn[d])), 0.01f);
        mn[d] = fsub(mn[d], s);
        mx[d] = fadd(mx[d], s);
    }
    // src/rtplugins/UniformGridAccStructBuilder.cpp:86-98
    float diag[3];
    for (int d = 0; d < 3; ++d) diag[d] = fsub(mx[d], mn[d]);
    const float V = fmul(fmul(diag[0], diag[1]), diag[2]);
    const int32_t kn = (int32_t)((uint32_t)k * (uint32_t)ntris);
    const float q = fdiv(__int2float_rn(kn), V);
    // powf(q, 1/3): the reference's C library powf is within one ulp of the
    // correctly rounded value and the device's single-precision powf within
    // a few ulps of it (CUDA's documented bound), so the resolution is
    // accepted only when ceil(d*f') is the same at both ends of a 16-ulp band
    // around the device's f (ceil(d*f') is monotonic in f'); otherwise the
    // host recomputes the parameters with the C library's powf.  (Evaluating
    // pow in double here made the last block's serial parameter step several
    // microseconds long: FP64 is a slow path on this GPU.)
    const float f = powf(q, 1.0f / 3.0f);
    const float fm = (f > 0.0f && isfinite(f)) ? __uint_as_float(__float_as_uint(f) - 16u) : f;
    const float fp = (f > 0.0f && isfinite(f)) ? __uint_as_float(__float_as_uint(f) + 16u) : f;
    uint32_t status = 0;
    int64_t ncells = 1;
    for (int d = 0; d < 3; ++d) {
        const float a = ceilf(fmul(diag[d], fm));
        const float b = ceilf(fmul(diag[d], f));
        const float c = ceilf(fmul(diag[d], fp));
        if (a != c) status |= ST_AMBIGUOUS;
        int32_t r = (b >= 1.0f && b < 2147483648.0f) ? (int32_t)b : 0;
        if (r <= 0) status |= ST_TOO_BIG;
        p->res[d] = r;
        ncells *= (r > 0 ? r : 1);
    }
    for (int d = 0; d < 3; ++d) {
        p->bmin[d] = mn[d];
        p->bmax[d] = mx[d];
        const float cs = fdiv(fsub(mx[d], mn[d]), __int2float_rn(p->res[d] > 0 ? p->res[d] : 1));
        p->cell[d] = cs;
        p->inv[d] = frcp(cs);
    }
    if (ncells >= INT32_MAX) status |= ST_TOO_BIG;
    // the occupancy bitmap shares the offsets capacity: words <= cells
    if (ncells + 1 > cell_cap) status |= ST_CELL_CAP;
    p->k = k;
    p->ncells = ncells;
    p->nrefs = 0;
    p->ntris = ntris;
    p->status = status;
    p->max_list = 0u;
    if (status) atomicOr(&w->sticky, status);
}

// clear = 0: a clear kernel on the record stream clears the offsets and the
// bitmap (a single-scene build with side streams), and this pass only
// reduces the box.
template <bool MULTI>
__global__ void __launch_bounds__(256) bbox_params_kernel(BuildArgs one, const BuildArgs* __restrict__ many, const int* __restrict__ first,
                       int ntasks, int clear) {
    pdl_begin();
    if (MULTI) {
        const int t = block_task(first, ntasks);
        const BuildArgs& a = many[t];
        const unsigned vbx = blockIdx.x - (unsigned)first[t], vgx = (unsigned)(first[t + 1] - first[t]);
        if (clear) zero_capacity(a.offsets, a.occ, a.cell_cap, vbx, vgx);
        bbox_params_body(a.verts, a.nverts, a.work, a.params, a.k, a.ntris, a.cell_cap, vbx, vgx);
    } else {
        const BuildArgs& a = one;
        if (clear) zero_capacity(a.offsets, a.occ, a.cell_cap, blockIdx.x, gridDim.x);
        bbox_params_body(a.verts, a.nverts, a.work, a.params, a.k, a.ntris, a.cell_cap, blockIdx.x, gridDim.x);
    }
}

// The offsets capacity and the bitmap cleared on the record stream, beside
// the box pass (nothing in it depends on the grid parameters).
__global__ void __launch_bounds__(256) clear_kernel(BuildArgs one) {
    pdl_begin();
    zero_capacity(one.offsets, one.occ, one.cell_cap, blockIdx.x, gridDim.x);
}

static __device__ __forceinline__ bool fatal(uint32_t s) {
    return (s & (ST_CELL_CAP | ST_AMBIGUOUS | ST_TOO_BIG)) != 0;
}

__device__ __forceinline__ void zero_offsets_body(int32_t* __restrict__ offsets, uint32_t* __restrict__ occ,
                                    const GridParams* __restrict__ p, unsigned vbx, unsigned vgx) {
    if (fatal(p->status)) return;
    if (occ) {
        const int64_t words = occ_words(p->res[0], p->res[1], p->res[2]);
        for (int64_t i = (int64_t)vbx * blockDim.x + threadIdx.x; i < words;
             i += (int64_t)vgx * blockDim.x)
            occ[i] = 0u;
    }
    const int64_t n = p->ncells + 1;
    const int64_t stride = (int64_t)vgx * blockDim.x * 4;
    for (int64_t i = ((int64_t)vbx * blockDim.x + threadIdx.x) * 4; i < n; i += stride) {
        if (i + 4 <= n && ((i & 3) == 0)) {
            reinterpret_cast<int4*>(offsets)[i >> 2] = make_int4(0, 0, 0, 0);
        } else {
            for (int64_t j = i; j < n && j < i + 4; ++j) offsets[j] = 0;
        }
    }
}

template <bool MULTI>
__global__ void zero_offsets_kernel(BuildArgs one, const BuildArgs* __restrict__ many, const int* __restrict__ first,
                       int ntasks) {
    pdl_begin();
    if (MULTI) {
        const int t = block_task(first, ntasks);
        const BuildArgs& a = many[t];
        zero_offsets_body(a.offsets, a.occ, a.params, blockIdx.x - (unsigned)first[t], (unsigned)(first[t + 1] - first[t]));
    } else {
        const BuildArgs& a = one;
        zero_offsets_body(a.offsets, a.occ, a.params, blockIdx.x, gridDim.x);
    }
}

// ---------------------------------------------------------------------------
// per-triangle cell ranges, expanded cooperatively by a warp
// ---------------------------------------------------------------------------
struct Lite {
    float bmin[3], inv[3];
    int32_t res[3];
};

__device__ __forceinline__ void load_lite(const GridParams* p, Lite& L) {
    for (int d = 0; d < 3; ++d) {
        L.bmin[d] = p->bmin[d];
        L.inv[d] = p->inv[d];
        L.res[d] = p->res[d];
    }
}

// Triangle box (v0, then expandBy v1, v2 with the reference's if / else-if)
// and its cell range, src/rtplugins/UniformGridAccStructBuilder.cpp:111-127.
__device__ __forceinline__ void tri_box_range(const Lite& L, const float3& v0, const float3& v1, const float3& v2,
                                              int32_t lo[3], int32_t hi[3]) {
    float bmn[3] = {v0.x, v0.y, v0.z}, bmx[3] = {v0.x, v0.y, v0.z};
    const float a1[3] = {v1.x, v1.y, v1.z}, a2[3] = {v2.x, v2.y, v2.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (a1[d] < bmn[d]) bmn[d] = a1[d];
        else if (a1[d] > bmx[d]) bmx[d] = a1[d];
        if (a2[d] < bmn[d]) bmn[d] = a2[d];
        else if (a2[d] > bmx[d]) bmx[d] = a2[d];
        lo[d] = world_to_voxel(bmn[d], L.bmin[d], L.inv[d]);
        hi[d] = world_to_voxel(bmx[d], L.bmin[d], L.inv[d]);
    }
}

// TriAccel::buildFrom (src/rtcore/Triangle.cpp:11-55): Wald's projection
// record, 48 bytes {k, n_u, n_v, n_d}, {b_nu, b_nv, b_d, 0}, {c_nu, c_nv,
// c_d, id}, every operation rounded once in float as the reference's code
// evaluates it (no contraction; IEEE division and reciprocal).  The trace
// evaluates the winning triangle's t / u / v from it exactly as
// RayTriIntersection::hitWald does, so a hit on the reference's triangle
// reports the reference's bits.
__device__ __forceinline__ float comp3(float x, float y, float z, uint32_t d) {
    return d == 0 ? x : (d == 1 ? y : z);
}
__device__ __forceinline__ void write_wald_record(float4* __restrict__ out, const float3& v0, const float3& v1,
                                                  const float3& v2, int32_t id) {
    const float bx = fsub(v2.x, v0.x), by = fsub(v2.y, v0.y), bz = fsub(v2.z, v0.z);
    const float cx = fsub(v1.x, v0.x), cy = fsub(v1.y, v0.y), cz = fsub(v1.z, v0.z);
    // normal = c x b
    const float nx = fsub(fmul(cy, bz), fmul(cz, by));
    const float ny = fsub(fmul(cz, bx), fmul(cx, bz));
    const float nz = fsub(fmul(cx, by), fmul(cy, bx));
    uint32_t k;
    if (vabs(nx) > vabs(ny) && vabs(nx) > vabs(nz)) k = 0;
    else if (vabs(ny) > vabs(nz)) k = 1;
    else k = 2;
    const uint32_t u = k == 2 ? 0 : k + 1, v = k == 0 ? 2 : k - 1;
    const float nk = comp3(nx, ny, nz, k), nu = comp3(nx, ny, nz, u), nv = comp3(nx, ny, nz, v);
    const float inv_nk = frcp(nk);
    const float nd = fadd(fadd(fmul(v0.x, fmul(nx, inv_nk)), fmul(v0.y, fmul(ny, inv_nk))), fmul(v0.z, fmul(nz, inv_nk)));
    const float bu = comp3(bx, by, bz, u), bv = comp3(bx, by, bz, v);
    const float cu = comp3(cx, cy, cz, u), cv = comp3(cx, cy, cz, v);
    const float v0u = comp3(v0.x, v0.y, v0.z, u), v0v = comp3(v0.x, v0.y, v0.z, v);
    const float inv_den = frcp(fsub(fmul(bu, cv), fmul(bv, cu)));
    out[0] = make_float4(__uint_as_float(k), fdiv(nu, nk), fdiv(nv, nk), nd);
    out[1] = make_float4(fmul(-bv, inv_den), fmul(bu, inv_den), fmul(fsub(fmul(bv, v0u), fmul(bu, v0v)), inv_den), 0.0f);
    out[2] = make_float4(fmul(cv, inv_den), fmul(-cu, inv_den), fmul(fsub(fmul(cu, v0v), fmul(cv, v0u)), inv_den),
                         __int_as_float(id));
}

__device__ __forceinline__ float3 load_vert(const float* __restrict__ verts, int32_t v) {
    const float* q = verts + 3 * (int64_t)v;
    return make_float3(__ldg(q), __ldg(q + 1), __ldg(q + 2));
}

// Enumerates every (cell, triangle) reference of the warp's 32 triangles, 32
// references per step, and calls emit(cell, tri, active) on every lane.
template <class Emit>
__device__ __forceinline__ void warp_expand(const Lite& L, const float* __restrict__ verts,
                                            const int32_t* __restrict__ idx, int64_t ntris, int64_t base,
                                            GridParams* p, BuildWork* w, Emit&& emit) {
    const int lane = threadIdx.x & 31;
    const int64_t t = base + lane;
    int32_t lo[3] = {0, 0, 0}, ext[3] = {1, 1, 1};
    uint32_t cnt = 0;
    if (t < ntris) {
        const int32_t i0 = __ldg(idx + 3 * t), i1 = __ldg(idx + 3 * t + 1), i2 = __ldg(idx + 3 * t + 2);
        const float3 v0 = load_vert(verts, i0), v1 = load_vert(verts, i1), v2 = load_vert(verts, i2);
        int32_t hi[3];
        tri_box_range(L, v0, v1, v2, lo, hi);
        bool ok = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            ok = ok && lo[d] >= 0 && hi[d] < L.res[d] && lo[d] <= hi[d];
            ext[d] = hi[d] - lo[d] + 1;
        }
        if (ok) {
            cnt = (uint32_t)ext[0] * (uint32_t)ext[1] * (uint32_t)ext[2];
        } else {
            raise_status(p, w, ST_BAD_RANGE);
            ext[0] = ext[1] = ext[2] = 1;
        }
    }
    unsigned long long incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
    }
    const unsigned long long total = __shfl_sync(FULL, incl, 31);
    const unsigned long long excl = incl - cnt;
    for (unsigned long long r0 = 0; r0 < total; r0 += 32) {
        const unsigned long long r = r0 + lane;
        const bool active = r < total;
        // owner lane j: smallest j with incl_j > r (exactly 5 halvings)
        int lo_ = 0, hi_ = 31;
#pragma unroll
        for (int s = 0; s < 5; ++s) {
            const int mid = (lo_ + hi_) >> 1;
            const unsigned long long im = __shfl_sync(FULL, incl, mid);
            if (im > r) hi_ = mid; else lo_ = mid + 1;
        }
        const int j = lo_;
        const unsigned long long ex_j = __shfl_sync(FULL, excl, j);
        const int32_t lx = __shfl_sync(FULL, lo[0], j), ly = __shfl_sync(FULL, lo[1], j),
                      lz = __shfl_sync(FULL, lo[2], j);
        const int32_t ex = __shfl_sync(FULL, ext[0], j), ey = __shfl_sync(FULL, ext[1], j);
        const uint32_t l = (uint32_t)(r - ex_j);
        const uint32_t rest = l / (uint32_t)ex;
        const int32_t x = lx + (int32_t)(l - rest * (uint32_t)ex);
        const int32_t y = ly + (int32_t)(rest % (uint32_t)ey);
        const int32_t z = lz + (int32_t)(rest / (uint32_t)ey);
        const int32_t cell = active ? (x + y * L.res[0] + z * L.res[0] * L.res[1]) : -1;
        emit(cell, (int32_t)(base + j), active);
    }
    if (lane == 0 && total) atomicAdd(reinterpret_cast<unsigned long long*>(&p->nrefs), total);
}

__device__ __forceinline__ void count_body(const float* __restrict__ verts, const int32_t* __restrict__ idx,
                                           int64_t ntris, GridParams* p, BuildWork* w,
                                           int32_t* __restrict__ counts, unsigned vbx, unsigned vgx) {
    if (fatal(p->status)) return;
    Lite L;
    load_lite(p, L);
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)vbx * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)vgx * blockDim.x) >> 5;
    // crowded cells: the block's additions gathered in a small
    // direct-mapped shared table (a slot taken by the first cell that maps
    // to it), flushed with one global atomic a slot at the end
    constexpr int kHot = 32;
    __shared__ int32_t hot_cell[kHot];
    __shared__ int32_t hot_cnt[kHot];
    if (threadIdx.x < kHot) {
        hot_cell[threadIdx.x] = -1;
        hot_cnt[threadIdx.x] = 0;
    }
    __syncthreads();
    for (int64_t base = warp * 32; base < ntris; base += nwarps * 32) {
        warp_expand(L, verts, idx, ntris, base, p, w, [&](int32_t cell, int32_t, bool active) {
            const unsigned peers = __match_any_sync(FULL, cell);
            const int leader = __ffs(peers) - 1;
            if (active && lane == leader) {
                const int slot = (int)(((uint32_t)cell * 2654435761u) >> 27);
                const int32_t old = atomicCAS(&hot_cell[slot], -1, cell);
                if (old == -1 || old == cell) atomicAdd(&hot_cnt[slot], __popc(peers));
                else atomicAdd(&counts[cell], __popc(peers));
            }
        });
    }
    __syncthreads();
    if (threadIdx.x < kHot && hot_cell[threadIdx.x] >= 0 && hot_cnt[threadIdx.x] > 0)
        atomicAdd(&counts[hot_cell[threadIdx.x]], hot_cnt[threadIdx.x]);
}

template <bool MULTI>
__global__ void __launch_bounds__(256) count_kernel(BuildArgs one, const BuildArgs* __restrict__ many, const int* __restrict__ first,
                       int ntasks) {
    pdl_begin();
    if (MULTI) {
        const int t = block_task(first, ntasks);
        const BuildArgs& a = many[t];
        count_body(a.verts, a.idx, a.ntris, a.params, a.work, a.offsets, blockIdx.x - (unsigned)first[t],
                   (unsigned)(first[t + 1] - first[t]));
    } else {
        const BuildArgs& a = one;
        count_body(a.verts, a.idx, a.ntris, a.params, a.work, a.offsets, blockIdx.x, gridDim.x);
    }
}

__device__ __forceinline__ void scatter_body(const float* __restrict__ verts, const int32_t* __restrict__ idx,
                                                      int64_t ntris, GridParams* p, int32_t* __restrict__ cursor,
                                                      int32_t* __restrict__ ids, unsigned vbx, unsigned vgx) {
    if (p->status & (ST_CELL_CAP | ST_AMBIGUOUS | ST_TOO_BIG | ST_REF_CAP)) return;
    Lite L;
    load_lite(p, L);
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)vbx * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)vgx * blockDim.x) >> 5;
    for (int64_t base = warp * 32; base < ntris; base += nwarps * 32) {
        const int64_t t = base + lane;
        int32_t lo[3] = {0, 0, 0}, ext[3] = {1, 1, 1};
        uint32_t cnt = 0;
        if (t < ntris) {
            const int32_t i0 = __ldg(idx + 3 * t), i1 = __ldg(idx + 3 * t + 1), i2 = __ldg(idx + 3 * t + 2);
            const float3 v0 = load_vert(verts, i0), v1 = load_vert(verts, i1), v2 = load_vert(verts, i2);
            int32_t hi[3];
            tri_box_range(L, v0, v1, v2, lo, hi);
            bool ok = true;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                ok = ok && lo[d] >= 0 && hi[d] < L.res[d] && lo[d] <= hi[d];
                ext[d] = hi[d] - lo[d] + 1;
            }
            if (ok) cnt = (uint32_t)ext[0] * (uint32_t)ext[1] * (uint32_t)ext[2];
            else ext[0] = ext[1] = ext[2] = 1;
        }
        unsigned long long incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        const unsigned long long total = __shfl_sync(FULL, incl, 31);
        const unsigned long long excl = incl - cnt;
        for (unsigned long long r0 = 0; r0 < total; r0 += 32) {
            const unsigned long long r = r0 + lane;
            const bool active = r < total;
            int lo_ = 0, hi_ = 31;
#pragma unroll
            for (int s = 0; s < 5; ++s) {
                const int mid = (lo_ + hi_) >> 1;
                const unsigned long long im = __shfl_sync(FULL, incl, mid);
                if (im > r) hi_ = mid; else lo_ = mid + 1;
            }
            const int j = lo_;
            const unsigned long long ex_j = __shfl_sync(FULL, excl, j);
            const int32_t lx = __shfl_sync(FULL, lo[0], j), ly = __shfl_sync(FULL, lo[1], j),
                          lz = __shfl_sync(FULL, lo[2], j);
            const int32_t ex = __shfl_sync(FULL, ext[0], j), ey = __shfl_sync(FULL, ext[1], j);
            const uint32_t l = (uint32_t)(r - ex_j);
            const uint32_t rest = l / (uint32_t)ex;
            const int32_t x = lx + (int32_t)(l - rest * (uint32_t)ex);
            const int32_t y = ly + (int32_t)(rest % (uint32_t)ey);
            const int32_t z = lz + (int32_t)(rest / (uint32_t)ey);
            const int32_t cell = active ? (x + y * L.res[0] + z * L.res[0] * L.res[1]) : -1;
            const unsigned peers = __match_any_sync(FULL, cell);
            const int leader = __ffs(peers) - 1;
            const int g = __popc(peers);
            const int rank = __popc(peers & ((1u << lane) - 1u));
            int32_t old = 0;
            if (active && lane == leader) old = atomicSub(&cursor[cell], g);
            old = __shfl_sync(FULL, old, leader);
            if (active) ids[old - g + rank] = (int32_t)(base + j);
        }
    }
}

template <bool MULTI>
__global__ void __launch_bounds__(256) scatter_kernel(BuildArgs one, const BuildArgs* __restrict__ many, const int* __restrict__ first,
                       int ntasks) {
    pdl_begin();
    if (MULTI) {
        const int t = block_task(first, ntasks);
        const BuildArgs& a = many[t];
        scatter_body(a.verts, a.idx, a.ntris, a.params, a.offsets, a.ids, blockIdx.x - (unsigned)first[t], (unsigned)(first[t + 1] - first[t]));
    } else {
        const BuildArgs& a = one;
        scatter_body(a.verts, a.idx, a.ntris, a.params, a.offsets, a.ids, blockIdx.x, gridDim.x);
    }
}

// ---------------------------------------------------------------------------
// scan of the per-cell counts (in place, inclusive), two phases: tile sums,
// then each tile scanned from the sum of the tiles before it
// ---------------------------------------------------------------------------
static constexpr int SCAN_THREADS = 256;
static constexpr int SCAN_ITEMS = kScanTile / SCAN_THREADS;  // 4 cells a thread: short chains, many blocks
static constexpr int SCAN_TILE = kScanTile;
static_assert(32 * SCAN_ITEMS < 256, "per-warp sort-queue counts fit 8 bits");

__device__ __forceinline__ int64_t block_sum_i64(int64_t v, int64_t* sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    int64_t s = 0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
        sh[32] = s;
    }
    __syncthreads();
    s = sh[32];
    __syncthreads();
    return s;
}

__device__ __forceinline__ void scan_reduce_body(const int32_t* __restrict__ counts,
                                                                   const GridParams* __restrict__ p,
                                                                   int64_t* __restrict__ tile_sums, unsigned vbx, unsigned vgx) {
    if (fatal(p->status)) return;
    const int64_t C = p->ncells;
    const int64_t ntiles = (C + SCAN_TILE - 1) / SCAN_TILE;
    __shared__ int64_t sh[33];
    for (int64_t tile = vbx; tile < ntiles; tile += vgx) {
        const int64_t b = tile * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
        int64_t s = 0;
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; ++i)
            if (b + i < C) s += counts[b + i];
        s = block_sum_i64(s, sh);
        if (threadIdx.x == 0) tile_sums[tile] = s;
    }
}

template <bool MULTI>
__global__ void __launch_bounds__(SCAN_THREADS) scan_reduce_kernel(BuildArgs one, const BuildArgs* __restrict__ many, const int* __restrict__ first,
                       int ntasks) {
    pdl_begin();
    if (MULTI) {
        const int t = block_task(first, ntasks);
        const BuildArgs& a = many[t];
        scan_reduce_body(a.offsets, a.params, a.tile_sums, blockIdx.x - (unsigned)first[t], (unsigned)(first[t + 1] - first[t]));
    } else {
        const BuildArgs& a = one;
        scan_reduce_body(a.offsets, a.params, a.tile_sums, blockIdx.x, gridDim.x);
    }
}

// Sort-queue class of a cell of n >= 2 entries (its BuildWork::nsort index).
__device__ __forceinline__ int sort_class(int32_t n) {
    return n <= SORT_TINY_MAX ? 0 : (n <= SORT_SMALL_MAX ? 3 : (n <= SORT_MED_MAX ? 1 : 2));
}

// In-place inclusive scan of each tile plus the sum of the tiles before it
// (each block adds those tile sums itself); queues cells that hold two or
// more triangles for the segmented sort.  The block of the last tile writes
// the reference total R = offsets[C] and checks it against the count pass
// and the capacities.
__device__ __forceinline__ void scan_down_body(int32_t* __restrict__ counts, GridParams* p,
                                                                 const int64_t* __restrict__ tile_sums,
                                                                 int64_t ref_cap,
                                                                 uint32_t* __restrict__ occ,
                                                                 BuildWork* w, int32_t* __restrict__ q_small,
                                                                 int32_t* __restrict__ q_med,
                                                                 int32_t* __restrict__ q_large, int64_t q_small_cap,
                                                                 int64_t q_med_cap, int64_t q_large_cap, unsigned vbx, unsigned vgx) {
    if (fatal(p->status)) return;
    const int64_t C = p->ncells;
    const int64_t ntiles = (C + SCAN_TILE - 1) / SCAN_TILE;
    __shared__ int64_t sh[9];
    __shared__ int64_t shs[33];
    __shared__ uint32_t wq[SCAN_THREADS / 32][4];   // per warp and class: count, then exclusive prefix
    __shared__ uint32_t qbase[4];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    // each block scans a contiguous run of tiles: the sum of the tiles
    // before its first one once, then a running total (summing every
    // earlier tile per tile costs tiles^2 / 2 reads: 34 M at 8.5 M cells)
    const int64_t per = (ntiles + vgx - 1) / vgx;
    const int64_t t0 = (int64_t)vbx * per, t1 = t0 + per < ntiles ? t0 + per : ntiles;
    if (t0 >= t1) return;
    int64_t before = 0;
#pragma unroll 4
    for (int64_t j = threadIdx.x; j < t0; j += blockDim.x) before += tile_sums[j];
    int64_t prefix = block_sum_i64(before, shs);
    for (int64_t tile = t0; tile < t1; ++tile) {
        const int64_t b = tile * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
        int32_t v[SCAN_ITEMS];
        int64_t s = 0;
        int32_t vmax = 0;
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; ++i) {
            v[i] = (b + i < C) ? counts[b + i] : 0;
            s += v[i];
            vmax = max(vmax, v[i]);
        }
        vmax = (int32_t)__reduce_max_sync(FULL, (unsigned)vmax);
        if (lane == 0 && vmax > 0) atomicMax(&p->max_list, (unsigned)vmax);
        int64_t x = s;
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(FULL, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) sh[wid] = x;
        __syncthreads();
        if (threadIdx.x == 0) {
            int64_t run = 0;
            for (int i = 0; i < SCAN_THREADS / 32; ++i) {
                int64_t t = sh[i];
                sh[i] = run;
                run += t;
            }
            sh[SCAN_THREADS / 32] = run;   // the tile's total
        }
        __syncthreads();
        int64_t run = prefix + sh[wid] + x - s;
        prefix += sh[SCAN_THREADS / 32];
        if (tile == ntiles - 1 && threadIdx.x == SCAN_THREADS - 1) {
            const int64_t R = run + s;   // the last thread's inclusive sum: the grand total
            if (R != p->nrefs) raise_status(p, w, ST_BAD_RANGE);
            if (R > ref_cap) raise_status(p, w, ST_REF_CAP);
            if (R >= INT32_MAX) raise_status(p, w, ST_TOO_BIG);
            counts[C] = (int32_t)R;
        }
        __syncthreads();
        if (occ && s > 0 && b < C) {
            // occupancy bits of this thread's 16 consecutive cells (one row
            // segment along x), one atomicOr per touched brick word
            const int32_t nx = p->res[0], ny = p->res[1];
            const int32_t bx = (nx + 3) >> 2, by = (ny + 3) >> 2;
            const int32_t b32 = (int32_t)b;   // < C, which fits int32 (else ST_TOO_BIG)
            int32_t cx = b32 % nx;
            const int32_t rest = b32 / nx;
            int32_t cy = rest % ny, cz = rest / ny;
            int64_t word = -1;
            uint32_t mask = 0u;
            for (int i = 0; i < SCAN_ITEMS && b + i < C; ++i) {
                if (v[i] > 0) {
                    const int64_t wi = (int64_t)(cx >> 2) + (int64_t)(cy >> 2) * bx + (int64_t)(cz >> 1) * bx * by;
                    if (wi != word) {
                        if (mask) atomicOr(&occ[word], mask);
                        word = wi;
                        mask = 0u;
                    }
                    mask |= occ_bit(cx, cy, cz);
                }
                if (++cx == nx) {
                    cx = 0;
                    if (++cy == ny) { cy = 0; ++cz; }
                }
            }
            if (mask) atomicOr(&occ[word], mask);
        }
        // cells to sort, by size class (the nsort index): four 8-bit counts
        // packed in one word (at most SCAN_ITEMS per thread, 32 x that per
        // warp), one warp scan, then the warps' totals scanned per class and
        // one atomicAdd per block and class.  Cells of 2..8 entries fill the
        // small queue from the front, cells of 9..32 from the back: a cell
        // in either holds two or more references, so together they number at
        // most R / 2 <= ref_cap / 2 < q_small_cap whenever R fits (R above
        // ref_cap raises ST_REF_CAP and the sorts skip the build)
        uint32_t packed = 0u;
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; ++i) {
            const int32_t n = v[i];
            if (b + i < C && n >= 2) packed += 1u << (8 * sort_class(n));
        }
        uint32_t incl = packed;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) {
#pragma unroll
            for (int k = 0; k < 4; ++k) wq[wid][k] = (incl >> (8 * k)) & 255u;
        }
        __syncthreads();
        if (threadIdx.x < 4) {
            uint32_t tot = 0u;
            for (int i = 0; i < SCAN_THREADS / 32; ++i) {
                const uint32_t t = wq[i][threadIdx.x];
                wq[i][threadIdx.x] = tot;
                tot += t;
            }
            qbase[threadIdx.x] = tot ? atomicAdd(&w->nsort[threadIdx.x], tot) : 0u;
        }
        __syncthreads();
        const uint32_t excl = incl - packed;
        uint32_t js = qbase[0] + wq[wid][0] + (excl & 255u);
        uint32_t jm = qbase[1] + wq[wid][1] + ((excl >> 8) & 255u);
        uint32_t jl = qbase[2] + wq[wid][2] + ((excl >> 16) & 255u);
        uint32_t jw = qbase[3] + wq[wid][3] + (excl >> 24);
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; ++i) {
            if (b + i < C) {
                run += v[i];
                counts[b + i] = (int32_t)run;
                const int32_t n = v[i];
                if (n >= 2) {
                    if (n <= SORT_TINY_MAX) {
                        if (js < q_small_cap) q_small[js] = (int32_t)(b + i);
                        else raise_status(p, w, ST_SORT_CAP);
                        ++js;
                    } else if (n <= SORT_SMALL_MAX) {
                        if (jw < q_small_cap) q_small[q_small_cap - 1 - jw] = (int32_t)(b + i);
                        else raise_status(p, w, ST_SORT_CAP);
                        ++jw;
                    } else if (n <= SORT_MED_MAX) {
                        if (jm < q_med_cap) q_med[jm] = (int32_t)(b + i);
                        else raise_status(p, w, ST_SORT_CAP);
                        ++jm;
                    } else {
                        if (jl < q_large_cap) q_large[jl] = (int32_t)(b + i);
                        else raise_status(p, w, ST_SORT_CAP);
                        ++jl;
                    }
                }
            }
        }
    }
}

template <bool MULTI>
__global__ void __launch_bounds__(SCAN_THREADS) scan_down_kernel(BuildArgs one, const BuildArgs* __restrict__ many, const int* __restrict__ first,
                       int ntasks) {
    pdl_begin();
    if (MULTI) {
        const int t = block_task(first, ntasks);
        const BuildArgs& a = many[t];
        scan_down_body(a.offsets, a.params, a.tile_sums, a.ref_cap, a.occ, a.work, a.q_small, a.q_med, a.q_large, a.q_small_cap, a.q_med_cap, a.q_large_cap, blockIdx.x - (unsigned)first[t], (unsigned)(first[t + 1] - first[t]));
    } else {
        const BuildArgs& a = one;
        scan_down_body(a.offsets, a.params, a.tile_sums, a.ref_cap, a.occ, a.work, a.q_small, a.q_med, a.q_large, a.q_small_cap, a.q_med_cap, a.q_large_cap, blockIdx.x, gridDim.x);
    }
}

// ---------------------------------------------------------------------------
// per-cell sorts (after scatter, offsets[c] .. offsets[c+1] is cell c's list)
// ---------------------------------------------------------------------------
static __device__ __forceinline__ bool sort_skip(const GridParams* p) {
    return (p->status & (ST_CELL_CAP | ST_AMBIGUOUS | ST_TOO_BIG | ST_REF_CAP | ST_SORT_CAP)) != 0;
}

__device__ __forceinline__ void sort_small_body(const int32_t* __restrict__ offsets, int32_t* __restrict__ ids,
                                                const int32_t* __restrict__ q, int64_t q_cap, const BuildWork* w,
                                                const GridParams* p, unsigned vbx, unsigned vgx) {
    if (sort_skip(p)) return;
    const int lane = threadIdx.x & 31;
    // cells of 2..8 entries (the queue's front): one per thread, a
    // 19-comparator network in registers
    const uint32_t nt = w->nsort[0];
    const int64_t tid = (int64_t)vbx * blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)vgx * blockDim.x;
    for (int64_t i = tid; i < nt; i += nthreads) {
        const int32_t c = q[i];
        const int32_t s = offsets[c], n = offsets[c + 1] - s;
        int32_t v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = k < n ? ids[s + k] : INT_MAX;
#define GRIDRT_CX(a, b) { const int32_t lo_ = min(v[a], v[b]), hi_ = max(v[a], v[b]); v[a] = lo_; v[b] = hi_; }
        GRIDRT_CX(0, 2) GRIDRT_CX(1, 3) GRIDRT_CX(4, 6) GRIDRT_CX(5, 7)
        GRIDRT_CX(0, 4) GRIDRT_CX(1, 5) GRIDRT_CX(2, 6) GRIDRT_CX(3, 7)
        GRIDRT_CX(0, 1) GRIDRT_CX(2, 3) GRIDRT_CX(4, 5) GRIDRT_CX(6, 7)
        GRIDRT_CX(2, 4) GRIDRT_CX(3, 5)
        GRIDRT_CX(1, 4) GRIDRT_CX(3, 6)
        GRIDRT_CX(1, 2) GRIDRT_CX(3, 4) GRIDRT_CX(5, 6)
#undef GRIDRT_CX
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < n) ids[s + k] = v[k];
    }
    // cells of 9..32 entries (the queue's back): one per warp, a bitonic
    // network over the lanes
    const uint32_t nw = w->nsort[3];
    const int64_t warp = tid >> 5, nwarps = nthreads >> 5;
    for (int64_t i = warp; i < nw; i += nwarps) {
        const int32_t c = q[q_cap - 1 - i];
        const int32_t cs = offsets[c], cn = offsets[c + 1] - cs;
        int32_t v = lane < cn ? ids[cs + lane] : INT_MAX;
#pragma unroll
        for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1) {
                const int32_t o = __shfl_xor_sync(FULL, v, j);
                const bool up = (lane & k) == 0;
                const bool lower = (lane & j) == 0;
                v = (lower == up) ? min(v, o) : max(v, o);
            }
        }
        if (lane < cn) ids[cs + lane] = v;
    }
}

template <bool MULTI>
__global__ void __launch_bounds__(256) sort_small_kernel(BuildArgs one, const BuildArgs* __restrict__ many, const int* __restrict__ first,
                       int ntasks) {
    pdl_begin();
    if (MULTI) {
        const int t = block_task(first, ntasks);
        const BuildArgs& a = many[t];
        sort_small_body(a.offsets, a.ids, a.q_small, a.q_small_cap, a.work, a.params, blockIdx.x - (unsigned)first[t], (unsigned)(first[t + 1] - first[t]));
    } else {
        const BuildArgs& a = one;
        sort_small_body(a.offsets, a.ids, a.q_small, a.q_small_cap, a.work, a.params, blockIdx.x, gridDim.x);
    }
}

// Cells of 33..256 entries: one warp per cell, a bitonic network over a
// power-of-two pad m = 32 V (V = 2, 4, 8 values per lane) held in registers:
// element e = 32 r + lane sits in register r of its lane, so strides below 32
// pair lanes (one shuffle per register) and strides of 32 and above pair
// registers of the same lane.  Every step is independent across the V
// registers, so a 256-entry list takes 36 steps of a few pipelined
// instructions instead of 144 dependent shared-memory round trips.
template <int V>
__device__ __forceinline__ void warp_bitonic_regs(int32_t* __restrict__ ids, int32_t s, int32_t n) {
    const int lane = threadIdx.x & 31;
    int32_t v[V];
#pragma unroll
    for (int r = 0; r < V; ++r) v[r] = 32 * r + lane < n ? ids[s + 32 * r + lane] : INT_MAX;
#pragma unroll
    for (int k = 2; k <= 32 * V; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j < 32) {
#pragma unroll
                for (int r = 0; r < V; ++r) {
                    const int32_t o = __shfl_xor_sync(FULL, v[r], j);
                    const bool up = ((32 * r + lane) & k) == 0;
                    const bool lower = (lane & j) == 0;
                    v[r] = (lower == up) ? min(v[r], o) : max(v[r], o);
                }
            } else {
                const int jr = j >> 5;
#pragma unroll
                for (int r = 0; r < V; ++r) {
                    if ((r & jr) == 0) {
                        const bool up = ((32 * r + lane) & k) == 0;
                        const int32_t lo = min(v[r], v[r | jr]), hi = max(v[r], v[r | jr]);
                        v[r] = up ? lo : hi;
                        v[r | jr] = up ? hi : lo;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < V; ++r)
        if (32 * r + lane < n) ids[s + 32 * r + lane] = v[r];
}

__device__ __forceinline__ void sort_medium_body(const int32_t* __restrict__ offsets,
                                                          int32_t* __restrict__ ids, const int32_t* __restrict__ q,
                                                          const BuildWork* w, const GridParams* p, unsigned vbx, unsigned vgx) {
    if (sort_skip(p)) return;
    const uint32_t nq = w->nsort[1];
    const int64_t warp = ((int64_t)vbx * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)vgx * blockDim.x) >> 5;
    for (int64_t i = warp; i < nq; i += nwarps) {
        const int32_t c = q[i];
        const int32_t s = offsets[c], n = offsets[c + 1] - s;
        if (n <= 64) warp_bitonic_regs<2>(ids, s, n);
        else if (n <= 128) warp_bitonic_regs<4>(ids, s, n);
        else warp_bitonic_regs<8>(ids, s, n);
    }
}

template <bool MULTI>
__global__ void __launch_bounds__(512) sort_medium_kernel(BuildArgs one, const BuildArgs* __restrict__ many, const int* __restrict__ first,
                       int ntasks) {
    pdl_begin();
    if (MULTI) {
        const int t = block_task(first, ntasks);
        const BuildArgs& a = many[t];
        sort_medium_body(a.offsets, a.ids, a.q_med, a.work, a.params, blockIdx.x - (unsigned)first[t], (unsigned)(first[t + 1] - first[t]));
    } else {
        const BuildArgs& a = one;
        sort_medium_body(a.offsets, a.ids, a.q_med, a.work, a.params, blockIdx.x, gridDim.x);
    }
}

// Cells above 256 entries, one block per cell: up to 4096 entries (and the
// dynamic shared memory's size) a bitonic network in shared memory; above,
// one shared-memory bit per id (per id chunk, from a scratch copy, when the
// scene has more triangles than the bitmap has bits), then the set bits
// written back in order.
// Lists above kSplitRefs entries of a single-scene build whose ids fit one
// bitmap span are sorted by sort_split_kernel, the rest by sort_large.
static constexpr int32_t kSplitRefs = SORT_BLOCK_MAX;
static constexpr int kSplitBlocks = 8;   // blocks of a list's cluster (the portable maximum)

__device__ __forceinline__ void sort_large_body(const int32_t* __restrict__ offsets,
                                                          int32_t* __restrict__ ids, int32_t* __restrict__ scratch,
                                                          const int32_t* __restrict__ q, const BuildWork* w,
                                                          const GridParams* p, int32_t bitmap_words, int64_t ntris,
                                                          unsigned vbx, unsigned vgx, bool skip_split = false) {
    if (sort_skip(p)) return;
    extern __shared__ uint32_t bm[];
    __shared__ int32_t sh_min[32], sh_max[32];
    __shared__ int32_t warp_tot[32];
    __shared__ int32_t base_sh;
    const uint32_t nq = w->nsort[2];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int bitonic_max = bitmap_words < SORT_BLOCK_MAX ? bitmap_words : SORT_BLOCK_MAX;
    for (int64_t qi = vbx; qi < nq; qi += vgx) {
        const int32_t c = q[qi];
        const int32_t s = offsets[c], n = offsets[c + 1] - s;
        if (skip_split && n > kSplitRefs) continue;
        if (n <= bitonic_max) {
            int32_t* a = reinterpret_cast<int32_t*>(bm);
            int m = 512;
            while (m < n) m <<= 1;
            for (int t = threadIdx.x; t < m; t += blockDim.x) a[t] = t < n ? ids[s + t] : INT_MAX;
            __syncthreads();
            for (int k = 2; k <= m; k <<= 1) {
                for (int j = k >> 1; j > 0; j >>= 1) {
                    for (int r = threadIdx.x; r < (m >> 1); r += blockDim.x) {
                        const int t = ((r & ~(j - 1)) << 1) | (r & (j - 1));
                        const int o = t + j;
                        const bool up = (t & k) == 0;
                        const int32_t x = a[t], y = a[o];
                        if ((x > y) == up) { a[t] = y; a[o] = x; }
                    }
                    __syncthreads();
                }
            }
            for (int t = threadIdx.x; t < n; t += blockDim.x) ids[s + t] = a[t];
            __syncthreads();
            continue;
        }
        // ids below one bitmap span (every id of a scene of at most
        // bitmap_words * 32 triangles): one pass straight from the list, no
        // copy and no range pass; otherwise copy to scratch and walk the id
        // range [min, max] a span at a time.  The global loads are issued
        // kSortLoads at a time per thread.
        constexpr int kSortLoads = 4;
        const int64_t span = (int64_t)bitmap_words * 32;
        const bool direct = ntris <= span;
        const int32_t* src = direct ? ids + s : scratch + s;
        int32_t mn = 0, mx = (int32_t)(ntris - 1);
        if (!direct) {
            mn = INT_MAX;
            mx = INT_MIN;
            for (int t0 = threadIdx.x; t0 < n; t0 += kSortLoads * blockDim.x) {
                int32_t v[kSortLoads];
#pragma unroll
                for (int u = 0; u < kSortLoads; ++u) {
                    const int t = t0 + u * blockDim.x;
                    v[u] = t < n ? ids[s + t] : 0;
                }
#pragma unroll
                for (int u = 0; u < kSortLoads; ++u) {
                    const int t = t0 + u * blockDim.x;
                    if (t < n) {
                        scratch[s + t] = v[u];
                        mn = min(mn, v[u]);
                        mx = max(mx, v[u]);
                    }
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                mn = min(mn, __shfl_xor_sync(FULL, mn, o));
                mx = max(mx, __shfl_xor_sync(FULL, mx, o));
            }
            if (lane == 0) { sh_min[wid] = mn; sh_max[wid] = mx; }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            if (!direct) {
                for (int i = 1; i < nw; ++i) { mn = min(mn, sh_min[i]); mx = max(mx, sh_max[i]); }
            }
            sh_min[0] = mn; sh_max[0] = mx;
            base_sh = 0;
        }
        __syncthreads();
        mn = sh_min[0];
        mx = sh_max[0];
        for (int64_t c0 = mn; c0 <= mx; c0 += span) {
            for (int i = threadIdx.x; i < bitmap_words; i += blockDim.x) bm[i] = 0u;
            __syncthreads();
            for (int t0 = threadIdx.x; t0 < n; t0 += kSortLoads * blockDim.x) {
                int32_t v[kSortLoads];
#pragma unroll
                for (int u = 0; u < kSortLoads; ++u) {
                    const int t = t0 + u * blockDim.x;
                    v[u] = t < n ? src[t] : 0;
                }
#pragma unroll
                for (int u = 0; u < kSortLoads; ++u) {
                    const int64_t d = (int64_t)v[u] - c0;
                    if (t0 + u * (int)blockDim.x < n && d >= 0 && d < span) atomicOr(&bm[d >> 5], 1u << (d & 31));
                }
            }
            __syncthreads();
            // each thread owns a contiguous run of words
            const int per = (bitmap_words + blockDim.x - 1) / blockDim.x;
            const int w0 = threadIdx.x * per, w1 = min(w0 + per, bitmap_words);
            int cnt = 0;
            for (int i = w0; i < w1; ++i) cnt += __popc(bm[i]);
            int x = cnt;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(FULL, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) warp_tot[wid] = x;
            __syncthreads();
            if (threadIdx.x == 0) {
                int run = 0;
                for (int i = 0; i < nw; ++i) { const int t = warp_tot[i]; warp_tot[i] = run; run += t; }
            }
            __syncthreads();
            int pos = s + base_sh + warp_tot[wid] + x - cnt;
            for (int i = w0; i < w1; ++i) {
                uint32_t bits = bm[i];
                while (bits) {
                    const int b = __ffs(bits) - 1;
                    bits &= bits - 1;
                    ids[pos++] = (int32_t)(c0 + (int64_t)i * 32 + b);
                }
            }
            __syncthreads();
            if (threadIdx.x == blockDim.x - 1) base_sh += warp_tot[wid] + x;
            __syncthreads();
        }
        __syncthreads();
    }
}

template <bool MULTI>
__global__ void __launch_bounds__(1024) sort_large_kernel(BuildArgs one, const BuildArgs* __restrict__ many, const int* __restrict__ first,
                       int ntasks, bool split) {
    pdl_begin();
    if (MULTI) {
        const int t = block_task(first, ntasks);
        const BuildArgs& a = many[t];
        sort_large_body(a.offsets, a.ids, a.scratch, a.q_large, a.work, a.params, a.bitmap_words, a.ntris, blockIdx.x - (unsigned)first[t], (unsigned)(first[t + 1] - first[t]));
    } else {
        const BuildArgs& a = one;
        sort_large_body(a.offsets, a.ids, a.scratch, a.q_large, a.work, a.params, a.bitmap_words, a.ntris, blockIdx.x,
                        gridDim.x, split);
    }
}

// A list above kSplitRefs entries, split by triangle id over the
// kSplitBlocks blocks of a thread-block cluster: block r owns the ids of
// slice r of [0, ntris) and a shared-memory bitmap of that slice.  Each
// block reads an eighth of the list and sets every entry's bit in the
// owning block's bitmap through distributed shared memory; after a cluster
// barrier each block counts its slice, reads the counts of the slices
// before it from their blocks, and writes its slice's ids in order.  The
// whole list has been read before the first barrier, so no entry is
// overwritten before it is read.  One block per list had sorted the
// longest list alone while the other SMs idled.
__global__ void __launch_bounds__(1024) sort_split_kernel(BuildArgs a) {
    pdl_begin();
    if (sort_skip(a.params)) return;
    extern __shared__ uint32_t sbm[];
    __shared__ int32_t warp_tot[32];
    __shared__ int32_t slice_total;
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int rank = (int)cl.block_rank();
    const unsigned cid = blockIdx.x / kSplitBlocks, ncl = gridDim.x / kSplitBlocks;
    const uint32_t nq = a.work->nsort[2];
    const int64_t slice = ((a.ntris + kSplitBlocks - 1) / kSplitBlocks + 31) & ~(int64_t)31;
    const int64_t lo = (int64_t)rank * slice;
    const int64_t hi = lo + slice < a.ntris ? lo + slice : a.ntris;
    const int words = hi > lo ? (int)((hi - lo + 31) >> 5) : 0;
    uint32_t* peer_bm[kSplitBlocks];
#pragma unroll
    for (int r = 0; r < kSplitBlocks; ++r) peer_bm[r] = cl.map_shared_rank(sbm, r);
    constexpr int kSortLoads = 4;
    for (int64_t qi = cid; qi < nq; qi += ncl) {
        const int32_t c = a.q_large[qi];
        const int32_t s = a.offsets[c], n = a.offsets[c + 1] - s;
        if (n <= kSplitRefs) continue;   // the same list on every block of the cluster
        for (int i = threadIdx.x; i < words; i += blockDim.x) sbm[i] = 0u;
        cl.sync();   // every bitmap cleared
        // this block's eighth of the list
        const int32_t part = (n + kSplitBlocks - 1) / kSplitBlocks;
        const int32_t p0 = rank * part, p1 = p0 + part < n ? p0 + part : n;
        for (int32_t t0 = p0 + (int32_t)threadIdx.x; t0 < p1; t0 += kSortLoads * (int32_t)blockDim.x) {
            int32_t v[kSortLoads];
#pragma unroll
            for (int u = 0; u < kSortLoads; ++u) {
                const int32_t t = t0 + u * (int32_t)blockDim.x;
                v[u] = t < p1 ? a.ids[s + t] : 0;
            }
#pragma unroll
            for (int u = 0; u < kSortLoads; ++u) {
                if (t0 + u * (int32_t)blockDim.x < p1) {
                    const int q = (int)((int64_t)v[u] / slice);
                    const int64_t d = (int64_t)v[u] - (int64_t)q * slice;
                    atomicOr(peer_bm[q] + (d >> 5), 1u << (d & 31));
                }
            }
        }
        cl.sync();   // every bit set, the whole list read
        // each thread owns a contiguous run of this block's words
        const int per = (words + blockDim.x - 1) / blockDim.x;
        const int w0 = (int)threadIdx.x * per < words ? (int)threadIdx.x * per : words;
        const int w1 = w0 + per < words ? w0 + per : words;
        int cnt = 0;
        for (int i = w0; i < w1; ++i) cnt += __popc(sbm[i]);
        int x = cnt;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(FULL, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[wid] = x;
        __syncthreads();
        if (threadIdx.x == 0) {
            int run = 0;
            for (int i = 0; i < nw; ++i) {
                const int t = warp_tot[i];
                warp_tot[i] = run;
                run += t;
            }
            slice_total = run;
        }
        cl.sync();   // every slice's count published
        int below = 0;
        for (int r = 0; r < rank; ++r) below += *cl.map_shared_rank(&slice_total, r);
        int pos = s + below + warp_tot[wid] + x - cnt;
        for (int i = w0; i < w1; ++i) {
            uint32_t bits = sbm[i];
            while (bits) {
                const int b = __ffs(bits) - 1;
                bits &= bits - 1;
                a.ids[pos++] = (int32_t)(lo + (int64_t)i * 32 + b);
            }
        }
        // no block clears its bitmap or republishes its count for the next
        // list while another may still read them
        cl.sync();
    }
}

// Triangle records in cell-list order: crec[3i..3i+2] = tris[3 ids[i] ..].
// One float4 a thread: thread q copies component q % 3 of the record of
// list entry q / 3, so a warp's stores cover 512 contiguous bytes (storing a
// whole record a thread left each store instruction 48 bytes apart a lane).
__device__ __forceinline__ void cell_records_body(const int32_t* __restrict__ ids, const float4* __restrict__ tris,
                                                  float4* __restrict__ crec, const GridParams* p, unsigned vbx,
                                                  unsigned vgx) {
    if (!crec || build_failed(p->status)) return;
    const int64_t Q = 3 * p->nrefs;
    const int64_t stride = (int64_t)vgx * blockDim.x;
    for (int64_t q = (int64_t)vbx * blockDim.x + threadIdx.x; q < Q; q += stride) {
        const int64_t i = q / 3;
        const int64_t t = __ldg(ids + i);
        crec[q] = __ldg(tris + 3 * t + (q - 3 * i));
    }
}

template <bool MULTI>
__global__ void __launch_bounds__(256) cell_records_kernel(BuildArgs one, const BuildArgs* __restrict__ many,
                                                           const int* __restrict__ first, int ntasks) {
    pdl_begin();
    if (MULTI) {
        const int t = block_task(first, ntasks);
        const BuildArgs& a = many[t];
        cell_records_body(a.ids, a.tris, a.crec, a.params, blockIdx.x - (unsigned)first[t],
                          (unsigned)(first[t + 1] - first[t]));
    } else {
        cell_records_body(one.ids, one.tris, one.crec, one.params, blockIdx.x, gridDim.x);
    }
}

// Triangle records, one triangle a thread: the trace's Moller-Trumbore record
// {v0, id}, {v1 - v0, 0}, {v2 - v0, 0} and, when the scene keeps them, the
// reference's TriAccel record.  Needs only the vertices and indices, so a
// single-scene build runs it on a stream of its own beside the grid passes.
__device__ __forceinline__ void records_body(const float* __restrict__ verts, const int32_t* __restrict__ idx,
                                             int64_t ntris, float4* __restrict__ tris, float4* __restrict__ wald,
                                             unsigned vbx, unsigned vgx) {
    const int64_t stride = (int64_t)vgx * blockDim.x;
    for (int64_t t = (int64_t)vbx * blockDim.x + threadIdx.x; t < ntris; t += stride) {
        const int32_t i0 = __ldg(idx + 3 * t), i1 = __ldg(idx + 3 * t + 1), i2 = __ldg(idx + 3 * t + 2);
        const float3 v0 = load_vert(verts, i0), v1 = load_vert(verts, i1), v2 = load_vert(verts, i2);
        tris[3 * t + 0] = make_float4(v0.x, v0.y, v0.z, __int_as_float((int32_t)t));
        tris[3 * t + 1] = make_float4(fsub(v1.x, v0.x), fsub(v1.y, v0.y), fsub(v1.z, v0.z), 0.0f);
        tris[3 * t + 2] = make_float4(fsub(v2.x, v0.x), fsub(v2.y, v0.y), fsub(v2.z, v0.z), 0.0f);
        if (wald) write_wald_record(wald + 3 * t, v0, v1, v2, (int32_t)t);
    }
}

template <bool MULTI>
__global__ void __launch_bounds__(256) records_kernel(BuildArgs one, const BuildArgs* __restrict__ many,
                                                      const int* __restrict__ first, int ntasks) {
    pdl_begin();
    if (MULTI) {
        const int t = block_task(first, ntasks);
        const BuildArgs& a = many[t];
        records_body(a.verts, a.idx, a.ntris, a.tris, a.wald, blockIdx.x - (unsigned)first[t],
                     (unsigned)(first[t + 1] - first[t]));
    } else {
        records_body(one.verts, one.idx, one.ntris, one.tris, one.wald, blockIdx.x, gridDim.x);
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
// Block counts per kernel for one task; the single-scene launch uses them as
// its grid sizes, the batch launch concatenates them per task.
void build_blocks(const BuildArgs& a, int sms, int out[kBuildKinds]) {
    auto clampi = [](int64_t v, int64_t hi) { return (int)(v < 1 ? 1 : (v > hi ? hi : v)); };
    // vertices to reduce, and the capacity to clear (4 cells a thread)
    const int64_t bbox_work = a.nverts > a.cell_cap / 4 ? a.nverts : a.cell_cap / 4;
    out[BK_BBOX] = clampi((bbox_work + 255) / 256, 4 * sms);
    out[BK_ZERO] = clampi((a.cell_cap / 4 + 255) / 256, 8 * sms);
    out[BK_TRI] = clampi((a.ntris + 255) / 256, 16 * sms);            // one warp per 32 triangles
    out[BK_TILE] = clampi((a.cell_cap + SCAN_TILE - 1) / SCAN_TILE, 8 * sms);
    out[BK_SSMALL] = clampi(a.cell_cap / 512 + 1, 8 * sms);
    out[BK_SMED] = clampi(a.cell_cap / 2048 + 1, 4 * sms);             // 16 warps a block, one cell a warp
    out[BK_SLARGE] = clampi(a.cell_cap / 16384 + 1, 2 * sms);
    out[BK_REFS] = a.crec ? clampi((3 * a.ref_cap + 255) / 256, 16 * sms) : 0;
    out[BK_RECS] = clampi((a.ntris + 255) / 256, 16 * sms);
}

// launch_k with a thread-block cluster of `cluster` blocks along x.
template <typename... KArgs, typename... Args>
static cudaError_t launch_cluster_k(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem,
                                    cudaStream_t st, unsigned cluster, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[2];
    unsigned na = 0;
    attr[na].id = cudaLaunchAttributeClusterDimension;
    attr[na].val.clusterDim.x = cluster;
    attr[na].val.clusterDim.y = 1;
    attr[na].val.clusterDim.z = 1;
    ++na;
#if GRIDRT_PDL
    attr[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[na].val.programmaticStreamSerializationAllowed = 1;
    ++na;
#endif
    cfg.attrs = attr;
    cfg.numAttrs = na;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

template <bool MULTI>
static void launch_build_impl(const BuildArgs& one, const BuildArgs* many, int ntasks, const BatchGrid& g,
                              bool skip_bbox, int bitmap_words, cudaStream_t st, const BuildFork* fork = nullptr) {
    count_launches(9);
    const int* f[kBuildKinds];
    for (int k = 0; k < kBuildKinds; ++k) f[k] = MULTI ? g.first[k] : nullptr;
    // the triangle records: on the record stream beside the whole build (it
    // starts after everything before the build on `st` -- the previous
    // frame's traces, which read the records -- and the build's end waits
    // for it), else first on `st`
    const bool rec_side = fork && fork->rec;
    const bool side_clear = rec_side && !MULTI && !skip_bbox;
    int bbox_blocks = g.total[BK_BBOX];
    if (rec_side) {
        cudaEventRecord(fork->rec_fork, st);
        cudaStreamWaitEvent(fork->rec, fork->rec_fork, 0);
        if (side_clear) {
            count_launches(1);
            launch_k(clear_kernel, g.total[BK_BBOX], 256, 0, fork->rec, one);
            cudaEventRecord(fork->rec_clear, fork->rec);
            // the box pass alone: four vertices a thread at least
            bbox_blocks = (int)((one.nverts + 1023) / 1024);
            bbox_blocks = bbox_blocks < 1 ? 1 : (bbox_blocks > 2 * one.num_sms ? 2 * one.num_sms : bbox_blocks);
        }
    }
    launch_k(records_kernel<MULTI>, g.total[BK_RECS], 256, 0, rec_side ? fork->rec : st, one, many, f[BK_RECS],
             ntasks);
    if (rec_side) cudaEventRecord(fork->rec_join, fork->rec);
    // the box pass also clears the offsets and the bitmap; host-resolved
    // parameters skip it and clear them on their own
    if (!skip_bbox)
        launch_k(bbox_params_kernel<MULTI>, bbox_blocks, 256, 0, st, one, many, f[BK_BBOX], ntasks,
                 side_clear ? 0 : 1);
    else
        launch_k(zero_offsets_kernel<MULTI>, g.total[BK_ZERO], 256, 0, st, one, many, f[BK_ZERO], ntasks);
    if (side_clear) cudaStreamWaitEvent(st, fork->rec_clear, 0);
    launch_k(count_kernel<MULTI>, g.total[BK_TRI], 256, 0, st, one, many, f[BK_TRI], ntasks);
    launch_k(scan_reduce_kernel<MULTI>, g.total[BK_TILE], SCAN_THREADS, 0, st, one, many, f[BK_TILE], ntasks);
    launch_k(scan_down_kernel<MULTI>, g.total[BK_TILE], SCAN_THREADS, 0, st, one, many, f[BK_TILE], ntasks);
    launch_k(scatter_kernel<MULTI>, g.total[BK_TRI], 256, 0, st, one, many, f[BK_TRI], ntasks);
    // the three size classes sort disjoint cells: with side streams they run
    // side by side, joined before the records pass reads the lists
    cudaStream_t sm = st, sl = st;
    if (fork) {
        cudaEventRecord(fork->fork, st);
        cudaStreamWaitEvent(fork->side[0], fork->fork, 0);
        cudaStreamWaitEvent(fork->side[1], fork->fork, 0);
        sm = fork->side[0];
        sl = fork->side[1];
    }
    launch_k(sort_small_kernel<MULTI>, g.total[BK_SSMALL], 256, 0, st, one, many, f[BK_SSMALL], ntasks);
    launch_k(sort_medium_kernel<MULTI>, g.total[BK_SMED], 512, 0, sm, one, many, f[BK_SMED], ntasks);
    // a single-scene build whose ids fit one bitmap span sorts its lists
    // above kSplitRefs entries with a cluster each, first (the longest work)
    bool split = !MULTI && one.ntris > 0 && one.ntris <= (int64_t)bitmap_words * 32;
    if (split) {
        const int clusters = one.num_sms / kSplitBlocks > 0 ? one.num_sms / kSplitBlocks : 1;
        const int64_t words = ((one.ntris + kSplitBlocks - 1) / kSplitBlocks + 31) / 32 + 1;
        if (launch_cluster_k(sort_split_kernel, (unsigned)(clusters * kSplitBlocks), 1024u, (size_t)words * 4, sl,
                             (unsigned)kSplitBlocks, one) == cudaSuccess) {
            count_launches(1);
        } else {
            // the cluster launch was refused: the block sort takes every list
            (void)cudaGetLastError();
            split = false;
        }
    }
    launch_k(sort_large_kernel<MULTI>, g.total[BK_SLARGE], 1024, (size_t)bitmap_words * 4, sl, one, many,
             f[BK_SLARGE], ntasks, split);
    if (fork) {
        cudaEventRecord(fork->join[0], sm);
        cudaEventRecord(fork->join[1], sl);
        cudaStreamWaitEvent(st, fork->join[0], 0);
        cudaStreamWaitEvent(st, fork->join[1], 0);
    }
    if (rec_side) cudaStreamWaitEvent(st, fork->rec_join, 0);
    if (g.total[BK_REFS] > 0) {
        count_launches(1);
        launch_k(cell_records_kernel<MULTI>, g.total[BK_REFS], 256, 0, st, one, many, f[BK_REFS], ntasks);
    }
}

void launch_build(const BuildArgs& a, cudaStream_t st, const BuildFork* fork) {
    BatchGrid g{};
    build_blocks(a, a.num_sms, g.total);
    launch_build_impl<false>(a, nullptr, 1, g, a.skip_bbox, a.bitmap_words, st, fork);
}

void launch_build_batch(const BuildArgs* d_tasks, int ntasks, const BatchGrid& g, int bitmap_words,
                        cudaStream_t st) {
    if (ntasks <= 0) return;
    BuildArgs dummy{};
    launch_build_impl<true>(dummy, d_tasks, ntasks, g, false, bitmap_words, st);
}

cudaError_t build_setup_attributes(int bitmap_words) {
    cudaError_t e = cudaFuncSetAttribute(sort_large_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         bitmap_words * 4);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(sort_large_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                bitmap_words * 4);
}

}  // namespace gridrt
