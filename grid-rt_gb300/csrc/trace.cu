// trace.cu -- launch counting, the batched tracer (many scenes, one persistent
// launch), two-level instancing and the device-side mesh deformation.
// The single-scene kernels are in trace_device.cuh and trace_{nearest,any,
// camera,frame}.cu.
#include "trace_device.cuh"

namespace gridrt {

static unsigned long long g_launches = 0;
void count_launches(int n) { __atomic_add_fetch(&g_launches, (unsigned long long)n, __ATOMIC_RELAXED); }
unsigned long long launches_so_far() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

// Task t owning flattened ray index f: the last task with first <= f.
__device__ __forceinline__ int find_task(const BatchTask* __restrict__ tasks, int ntasks, long long f) {
    int lo = 0, hi = ntasks - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tasks[mid].first <= f) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Lane refill inside one batch task (TraceIO::refill > 0): the warp draws
// 32-ray chunks from the flattened counter and hands their rays to idle
// lanes while the chunks belong to its task, so scene and mode stay
// warp-uniform; a chunk of a later task ends the task here once its rays
// are finished and is returned (or a value >= total at the end).
template <int MODE, int ER>
__device__ __forceinline__ unsigned long long trace_task_refill(const SParams& P, const SceneView& s,
                                                                const TraceIO& io, Lane& L, long long tfirst,
                                                                unsigned long long chunk, long long total,
                                                                uint32_t& cells, uint32_t& tests,
                                                                uint32_t& started) {
    const int lane = threadIdx.x & 31;
    long long pb = (long long)chunk - tfirst;                 // task-local rays not yet started: [pb, pe)
    long long pe = pb + 32 < io.n ? pb + 32 : io.n;
    unsigned long long next = ~0ull;                          // a claimed chunk past this task
    bool active = false;
    int32_t heavy = io.heavy, work_cap = kNoHeavy;
    for (;;) {
        const unsigned idle = __ballot_sync(FULL, !active);
        const int nidle = __popc(idle);
        const bool room = nidle >= io.refill || idle == FULL;
        if (pb >= pe && next == ~0ull && room) {
            unsigned long long nb = 0;
            if (lane == 0) nb = atomicAdd(io.counter, 32ull);
            nb = __shfl_sync(FULL, nb, 0);
            if ((long long)nb < tfirst + io.n) {
                pb = (long long)nb - tfirst;
                pe = pb + 32 < io.n ? pb + 32 : io.n;
            } else {
                next = nb;
            }
        }
        if (pb < pe && room) {
            const int take = (long long)nidle < pe - pb ? nidle : (int)(pe - pb);
            if (!active) {
                const int rank = __popc(idle & ((1u << lane) - 1u));
                if (rank < take) {
                    L.ray = (int32_t)(pb + rank);
                    heavy = io.heavy;
                    work_cap = heavy < kNoHeavy / (kHeavyWorkMult + 1) && kHeavyWorkMult > 0 ? heavy * kHeavyWorkMult
                                                                                             : kNoHeavy;
                    ++started;
                    if (start_ray<MODE>(P, io, L, L.ray)) {
                        active = true;
                    } else {
                        if (L.id != -2) L.id = -1;
                        finish_ray<MODE>(io, P, s, L);
                    }
                }
            }
            pb += take;
        }
        if (!__any_sync(FULL, active)) {
            if (pb >= pe && next != ~0ull) return next;
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
        if (fin) {
            finish_ray<MODE>(io, P, s, L);
            active = false;
        }
    }
}

// Many (scene, ray batch) tasks in one persistent launch.  Task t owns the
// 32-aligned index range [first, first + n) of one flattened ray space, so a
// 32-ray claim always falls inside one task: scene and mode are warp-uniform.
template <int ER, bool REFILL>
__global__ void __launch_bounds__(128, GRIDRT_TRACE_MIN_BLOCKS)
    trace_batch_kernel(const BatchScene* __restrict__ scenes, int nscenes, const BatchTask* __restrict__ tasks,
                       int ntasks, long long total, unsigned long long* counter, int2* defer, int32_t defer_cap,
                       int32_t heavy, int32_t refill) {
    pdl_begin();
    __shared__ SParams P[kMaxBatchScenes];
    for (int i = threadIdx.x; i < nscenes; i += blockDim.x) fill_sparams(scenes[i].view.params, P[i]);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    Lane L;
    uint32_t cells = 0, tests = 0, started = 0;
    unsigned long long b = 0;
    if (lane == 0) b = atomicAdd(counter, 32ull);
    b = __shfl_sync(FULL, b, 0);
    while ((long long)b < total) {
        const BatchTask T = tasks[find_task(tasks, ntasks, (long long)b)];
        const SceneView V = scenes[T.scene].view;
        TraceIO io{};
        io.rays = T.rays;
        io.n = T.n;
        io.counter = counter;
        io.defer = defer;
        io.defer_cap = defer_cap;
        io.heavy = defer ? heavy : kNoHeavy;
        io.defer_base = (int32_t)T.first;
        io.refill = refill;
        if (REFILL) {
            if (T.mode == MODE_ANY) {
                io.occ = static_cast<uint8_t*>(T.out);
                b = trace_task_refill<MODE_ANY, ER>(P[T.scene], V, io, L, T.first, b, total, cells, tests, started);
            } else {
                io.hits = static_cast<int4*>(T.out);
                b = trace_task_refill<MODE_NEAREST, ER>(P[T.scene], V, io, L, T.first, b, total, cells, tests,
                                                        started);
            }
            continue;
        }
        const long long base = (long long)b - T.first;
        if (T.mode == MODE_ANY) {
            io.occ = static_cast<uint8_t*>(T.out);
            trace_batch32<MODE_ANY, ER>(P[T.scene], V, io, L, base, cells, tests, started);
        } else {
            io.hits = static_cast<int4*>(T.out);
            trace_batch32<MODE_NEAREST, ER>(P[T.scene], V, io, L, base, cells, tests, started);
        }
        if (lane == 0) b = atomicAdd(counter, 32ull);
        b = __shfl_sync(FULL, b, 0);
    }
}

// Warp-per-ray pass over the rays a batch launch deferred (flattened
// indices); each group resolves its own task, scene and mode.
template <int G>
__global__ void __launch_bounds__(128) trace_wide_batch_kernel(const BatchScene* __restrict__ scenes, int nscenes,
                                                               const BatchTask* __restrict__ tasks, int ntasks,
                                                               unsigned long long* counter,
                                                               const int2* __restrict__ defer, int32_t defer_cap) {
    pdl_begin();
    __shared__ SParams P[kMaxBatchScenes];
    for (int i = threadIdx.x; i < nscenes; i += blockDim.x) fill_sparams(scenes[i].view.params, P[i]);
    __syncthreads();
    const int lane = threadIdx.x & 31, gl = lane & (G - 1), grp = lane / G;
    unsigned long long nd = counter[1];
    if (nd > (unsigned long long)defer_cap) nd = (unsigned long long)defer_cap;
    uint32_t cells = 0, tests = 0;
    for (;;) {
        unsigned long long j0 = 0;
        if (lane == 0) j0 = atomicAdd(counter + 2, (unsigned long long)(32 / G));
        j0 = __shfl_sync(FULL, j0, 0);
        if (j0 >= nd) break;
        const unsigned long long j = j0 + grp;
        const bool valid = j < nd;
        bool done = true, any = false;
        int scene = 0;
        Lane L;
        L.best = kFltMax;
        L.id = -1;
        TraceIO io{};
        if (valid) {
            const int2 d = __ldg(defer + j);
            const BatchTask T = tasks[find_task(tasks, ntasks, (long long)d.x)];
            scene = T.scene;
            any = T.mode == MODE_ANY;
            io.rays = T.rays;
            io.n = T.n;
            L.ray = (int32_t)((long long)d.x - T.first);
            if (any) {
                io.occ = static_cast<uint8_t*>(T.out);
                done = !start_ray<MODE_ANY>(P[scene], io, L, L.ray);
            } else {
                io.hits = static_cast<int4*>(T.out);
                done = !start_ray<MODE_NEAREST>(P[scene], io, L, L.ray);
            }
            if (done) {
                if (L.id != -2) L.id = -1;
            } else {
                resume_at(P[scene], L, d.y);
            }
        }
        const SceneView V = scenes[scene].view;
        wide_walk<G>(P[scene], V, L, done, any, cells, tests);
        if (valid && gl == 0) {
            if (any) finish_ray<MODE_ANY>(io, P[scene], V, L);
            else finish_ray<MODE_NEAREST>(io, P[scene], V, L);
        }
    }
}

// ---------------------------------------------------------------------------
// two-level instancing: IAccStruct::traceNearestInstance
// (src/rtcore/IAccStruct.cpp:26-72).  The ray is clipped against the scene
// box (union of the instances' world boxes); then, instance by instance in
// order, the ray taken to the instance's local space (same tnear / tfar,
// direction not renormalised, so t is the same in both spaces) walks that
// instance's grid starting from the best distance so far: a later instance
// wins only with a strictly closer hit.  Matrix rows are applied as
// x' = ((m0 x + m1 y) + m2 z) + m3, one rounding per operation.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void xf_point(const float* m, float x, float y, float z, float& ox, float& oy, float& oz) {
    ox = fadd(fadd(fadd(fmul(m[0], x), fmul(m[1], y)), fmul(m[2], z)), m[3]);
    oy = fadd(fadd(fadd(fmul(m[4], x), fmul(m[5], y)), fmul(m[6], z)), m[7]);
    oz = fadd(fadd(fadd(fmul(m[8], x), fmul(m[9], y)), fmul(m[10], z)), m[11]);
}

__device__ __forceinline__ void xf_dir(const float* m, float x, float y, float z, float& ox, float& oy, float& oz) {
    ox = fadd(fadd(fmul(m[0], x), fmul(m[1], y)), fmul(m[2], z));
    oy = fadd(fadd(fmul(m[4], x), fmul(m[5], y)), fmul(m[6], z));
    oz = fadd(fadd(fmul(m[8], x), fmul(m[9], y)), fmul(m[10], z));
}

__global__ void instances_prep_kernel(const InstanceRec* __restrict__ recs, int ninst, SParams* __restrict__ sp) {
    pdl_begin();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ninst; i += gridDim.x * blockDim.x)
        fill_sparams(recs[i].view.params, sp[i]);
}

template <int MODE, int ER>
__global__ void __launch_bounds__(128) trace_instances_kernel(const InstanceRec* __restrict__ recs,
                                                              const SParams* __restrict__ sp, int ninst,
                                                              InstanceBox box, TraceIO io, int32_t* inst_out) {
    pdl_begin();
    __shared__ SParams Pw[4];
    const int lane = threadIdx.x & 31;
    SParams& P = Pw[threadIdx.x >> 5];
    uint32_t cells = 0, tests = 0, started = 0;
    for (;;) {
        unsigned long long b = 0;
        if (lane == 0) b = atomicAdd(io.counter, 32ull);
        b = __shfl_sync(FULL, b, 0);
        if ((long long)b >= io.n) break;
        const long long r = (long long)b + lane;
        bool alive = r < io.n, noray = false;
        float wo[3] = {0.f, 0.f, 0.f}, wd[3] = {1.f, 1.f, 1.f};
        float tn = 0.f, tf = 0.f, tmax = 0.f;
        if (alive) {
            ++started;
            const float4 a = __ldg(io.rays + 2 * r), c = __ldg(io.rays + 2 * r + 1);
            wo[0] = a.x; wo[1] = a.y; wo[2] = a.z;
            wd[0] = c.x; wd[1] = c.y; wd[2] = c.z;
            tn = a.w;
            tf = tmax = c.w;
            if (MODE == MODE_ANY && tf < 0.0f) {
                noray = true;
                alive = false;
            } else {
                // Ray::update + AabbIntersection::clipRay on the scene box
                float rn = tn, rf = tf;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const float inv = frcp(wd[d]);
                    const float t0 = fmul(fsub(box.bmin[d], wo[d]), inv), t1 = fmul(fsub(box.bmax[d], wo[d]), inv);
                    rn = vmax(rn, vmin(t0, t1));
                    rf = vmin(rf, vmax(t0, t1));
                }
                if (rn > rf) alive = false;
                tn = rn;
                tf = rf;
            }
        }
        float gbest = kFltMax;
        int32_t gid = -1, ginst = -1;
        for (int i = 0; i < ninst; ++i) {
            if (!__any_sync(FULL, alive)) break;
            __syncwarp();
            {
                const uint32_t* src = reinterpret_cast<const uint32_t*>(sp + i);
                uint32_t* dst = reinterpret_cast<uint32_t*>(&P);
                for (int w = lane; w < (int)(sizeof(SParams) / 4); w += 32) dst[w] = __ldg(src + w);
            }
            __syncwarp();
            const InstanceRec* R = recs + i;
            Lane L;
            bool active = alive && !P.failed && !__ldg(&R->skip);
            if (active) {
                float m[12];
#pragma unroll
                for (int k = 0; k < 12; ++k) m[k] = __ldg(&R->xf[k]);
                xf_point(m, wo[0], wo[1], wo[2], L.ox, L.oy, L.oz);
                xf_dir(m, wd[0], wd[1], wd[2], L.dx, L.dy, L.dz);
                active = setup_ray(P, L, tn, tf);
                L.tmax = tmax;
                if (MODE == MODE_NEAREST) L.best = gbest;
            }
            const int32_t* offs = R->view.offsets;
            const int32_t* ids = R->view.ids;
            const float4* tris = R->view.tris;
            const uint32_t* occ = R->view.occ;
            const float4* crec = R->view.crec;
            while (__any_sync(FULL, active)) {
                if (active && advance<MODE, ER>(P, L, offs, ids, tris, R->view.wald, occ, crec, kNoHeavy, kNoHeavy, cells, tests)) {
                    active = false;
                    if (L.id >= 0) {
                        // the next instance compares against the exact
                        // distance (the walk may have accepted its hit on
                        // Moller-Trumbore's t)
                        gbest = wald_f_of(L, L.id, R->view.wald);
                        gid = L.id;
                        ginst = i;
                        if (MODE == MODE_ANY) alive = false;   // occluded
                    }
                }
            }
        }
        if (r < io.n) {
            if (MODE == MODE_ANY) {
                io.occ[r] = noray ? 2 : (gid >= 0 ? 1 : 0);
            } else {
                int4 h = make_int4(-1, 0, 0, 0);
                if (gid >= 0) {
                    // reported values in the winning instance's space
                    const InstanceRec* R = recs + ginst;
                    float m[12];
#pragma unroll
                    for (int k = 0; k < 12; ++k) m[k] = __ldg(&R->xf[k]);
                    Lane L;
                    xf_point(m, wo[0], wo[1], wo[2], L.ox, L.oy, L.oz);
                    xf_dir(m, wd[0], wd[1], wd[2], L.dx, L.dy, L.dz);
                    L.id = gid;
                    L.best = gbest;
                    h = wald_hit(R->view.wald, L);
                }
                io.hits[r] = h;
                if (inst_out) inst_out[r] = ginst;
            }
        }
    }
    if (io.ctr) flush_counters(io.ctr, started, cells, tests);
}

template <int MODE, int ER>
static void launch_instances_er(const InstanceRec* recs, const SParams* sp, int ninst, const InstanceBox& box,
                                const TraceIO& io, int32_t* inst_out, const TraceTuning& tune, int num_sms,
                                cudaStream_t st) {
    static int per_sm = 0;
    if (per_sm == 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, trace_instances_kernel<MODE, ER>, 128, 0);
        per_sm = b > 0 ? b : 1;
    }
    long long blocks = (io.n + 127) / 128;
    if (tune.persistent) blocks = blocks < (long long)per_sm * num_sms ? blocks : (long long)per_sm * num_sms;
    if (blocks < 1) blocks = 1;
    if (blocks > 0x7fffffffLL) blocks = 0x7fffffffLL;
    trace_instances_kernel<MODE, ER><<<(int)blocks, 128, 0, st>>>(recs, sp, ninst, box, io, inst_out);
}

size_t instance_params_bytes(int ninst) { return sizeof(SParams) * (size_t)(ninst > 0 ? ninst : 1); }

void launch_trace_instances(const InstanceRec* recs, void* d_params, int ninst, const InstanceBox& box,
                            const float4* rays, int64_t n, int4* hits, int32_t* inst_out, uint8_t* occ, int mode,
                            TraceCounters* ctr, unsigned long long* counter, const TraceTuning& tune, int num_sms,
                            cudaStream_t st) {
    if (n <= 0 || ninst <= 0) return;
    count_launches(2);
    SParams* sp = static_cast<SParams*>(d_params);
    instances_prep_kernel<<<(ninst + 127) / 128, 128, 0, st>>>(recs, ninst, sp);
    cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st);
    TraceIO io{};
    io.rays = rays;
    io.hits = hits;
    io.occ = occ;
    io.n = n;
    io.counter = counter;
    io.ctr = ctr;
    io.heavy = kNoHeavy;
    const int er = tune.empty_run;
    if (mode == MODE_ANY) {
        if (er <= 2) launch_instances_er<MODE_ANY, 2>(recs, sp, ninst, box, io, inst_out, tune, num_sms, st);
        else if (er <= 4) launch_instances_er<MODE_ANY, 4>(recs, sp, ninst, box, io, inst_out, tune, num_sms, st);
        else launch_instances_er<MODE_ANY, 8>(recs, sp, ninst, box, io, inst_out, tune, num_sms, st);
    } else {
        if (er <= 2) launch_instances_er<MODE_NEAREST, 2>(recs, sp, ninst, box, io, inst_out, tune, num_sms, st);
        else if (er <= 4) launch_instances_er<MODE_NEAREST, 4>(recs, sp, ninst, box, io, inst_out, tune, num_sms, st);
        else launch_instances_er<MODE_NEAREST, 8>(recs, sp, ninst, box, io, inst_out, tune, num_sms, st);
    }
}

__global__ void deform_kernel(const float* __restrict__ base, const float* __restrict__ nrm, float* __restrict__ out,
                              int64_t nverts, float amp, float freq, float phase) {
    pdl_begin();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nverts; i += stride) {
        const float px = base[3 * i], py = base[3 * i + 1], pz = base[3 * i + 2];
        const float s = amp * sinf(freq * px + phase);
        out[3 * i] = px + s * nrm[3 * i];
        out[3 * i + 1] = py + s * nrm[3 * i + 1];
        out[3 * i + 2] = pz + s * nrm[3 * i + 2];
    }
}

template <int ER>
static void launch_batch_er(const BatchScene* scenes, int nscenes, const BatchTask* tasks, int ntasks, long long total,
                            const TraceSlot& slot, int32_t heavy, int32_t refill, int num_sms, cudaStream_t st) {
    static int per_sm = 0;
    if (per_sm == 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, trace_batch_kernel<ER, false>, 128, 0);
        per_sm = b > 0 ? b : 1;
    }
    long long blocks = (total + 127) / 128;
    blocks = blocks < (long long)per_sm * num_sms ? blocks : (long long)per_sm * num_sms;
    if (blocks < 1) blocks = 1;
    if (refill > 0)
        launch_k(trace_batch_kernel<ER, true>, (unsigned)blocks, 128, 0, st, scenes, nscenes, tasks, ntasks, total,
                 slot.ctr, heavy > 0 ? slot.defer : nullptr, slot.defer_cap, heavy, refill);
    else
        launch_k(trace_batch_kernel<ER, false>, (unsigned)blocks, 128, 0, st, scenes, nscenes, tasks, ntasks, total,
                 slot.ctr, heavy > 0 ? slot.defer : nullptr, slot.defer_cap, heavy, refill);
}

template <int G>
static void launch_wide_batch(const BatchScene* scenes, int nscenes, const BatchTask* tasks, int ntasks,
                              const TraceSlot& slot, int num_sms, cudaStream_t st) {
    static int per_sm = 0;
    if (per_sm == 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, trace_wide_batch_kernel<G>, 128, 0);
        per_sm = b > 0 ? b : 1;
    }
    launch_k(trace_wide_batch_kernel<G>, (unsigned)(per_sm * num_sms), 128, 0, st, scenes, nscenes, tasks, ntasks,
             slot.ctr, slot.defer, slot.defer_cap);
}

void launch_trace_batch(const BatchScene* scenes, int nscenes, const BatchTask* tasks, int ntasks, long long total,
                        const TraceSlot& slot, const TraceTuning& tune, int num_sms, cudaStream_t st) {
    if (total <= 0 || ntasks <= 0) return;
    // deferred entries are int32 flattened indices
    const bool defer = tune.heavy_cell > 0 && slot.defer && slot.defer_cap > 0 && total <= 0x7fffffffLL;
    const int32_t heavy = defer ? tune.heavy_cell : 0;
    count_launches(defer ? 2 : 1);
    cudaMemsetAsync(slot.ctr, 0, 3 * sizeof(unsigned long long), st);
    if (tune.empty_run <= 2) launch_batch_er<2>(scenes, nscenes, tasks, ntasks, total, slot, heavy, refill_for(tune, 0), num_sms, st);
    else if (tune.empty_run <= 4) launch_batch_er<4>(scenes, nscenes, tasks, ntasks, total, slot, heavy, refill_for(tune, 0), num_sms, st);
    else if (tune.empty_run <= 8) launch_batch_er<8>(scenes, nscenes, tasks, ntasks, total, slot, heavy, refill_for(tune, 0), num_sms, st);
    else launch_batch_er<16>(scenes, nscenes, tasks, ntasks, total, slot, heavy, refill_for(tune, 0), num_sms, st);
    if (defer) {
        if (tune.heavy_lanes <= 4) launch_wide_batch<4>(scenes, nscenes, tasks, ntasks, slot, num_sms, st);
        else if (tune.heavy_lanes <= 8) launch_wide_batch<8>(scenes, nscenes, tasks, ntasks, slot, num_sms, st);
        else if (tune.heavy_lanes <= 16) launch_wide_batch<16>(scenes, nscenes, tasks, ntasks, slot, num_sms, st);
        else launch_wide_batch<32>(scenes, nscenes, tasks, ntasks, slot, num_sms, st);
    }
}

void launch_deform(const float* base, const float* normals, float* out, int64_t nverts, float amp, float freq,
                   float phase, cudaStream_t st) {
    if (nverts <= 0) return;
    count_launches(1);
    int64_t blocks = (nverts + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    launch_k(deform_kernel, (unsigned)blocks, 256, 0, st, base, normals, out, nverts, amp, freq, phase);
}

}  // namespace gridrt
