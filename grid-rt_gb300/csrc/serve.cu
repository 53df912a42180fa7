// serve.cu -- continuous-batching request loop over resident scenes.
//
// The reference has no serving path; this is the request-level driver around
// the batched tracer.  Requests (scene, closest / any-hit, host rays) arrive at
// given times.  The loop, in real time:
//   * moves arrived requests to a FIFO of pending requests;
//   * admits pending requests into the next step while a device pool of
//     fixed size has room for their rays and results (admission by memory);
//   * launches a step -- ray uploads, one persistent trace launch over all of
//     the step's requests (each its own task), result downloads -- on its own
//     stream, with up to max_in_flight steps on the GPU at once, so requests
//     that arrive while earlier steps run join the next step;
//   * records each request's completion when its step's event has fired, and
//     returns pool memory in step order.
// plain = 1 serves one request at a time through the single-scene trace
// kernel (upload, trace, download, wait), the per-request baseline.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <string>
#include <thread>
#include <vector>

#include "scene.h"

using namespace gridrt;

namespace {

constexpr int kMaxStepTasks = 8192;
constexpr int kMaxInFlight = 8;

inline int64_t align256(int64_t b) { return (b + 255) / 256 * 256; }

struct Step {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    BatchTask* h_tasks = nullptr;   // pinned
    BatchTask* d_tasks = nullptr;
    unsigned long long* d_counter = nullptr;   // ray claims, deferred rays, deferred claims
    int2* d_defer = nullptr;                   // deferred-ray queue of the step's launch
    std::vector<int64_t> reqs;
    int64_t pool_end = 0;           // pool head after this step's allocations
    bool busy = false;
    bool reported = false;
};

// FIFO ring over [0, cap): allocations at the head, released in order.
struct Ring {
    int64_t cap = 0, head = 0, tail = 0, used = 0;
    bool alloc(int64_t bytes, int64_t* off) {
        if (bytes > cap) return false;
        if (head >= tail && used < cap) {       // free space: [head, cap) and [0, tail)
            if (cap - head >= bytes) {
                *off = head;
                head += bytes;
                used += bytes;
                return true;
            }
            if (tail >= bytes) {                // wrap: the gap at the end is wasted until released
                used += cap - head;
                *off = 0;
                head = bytes;
                used += bytes;
                return true;
            }
            return false;
        }
        if (head < tail && tail - head >= bytes) {
            *off = head;
            head += bytes;
            used += bytes;
            return true;
        }
        return false;
    }
    void release_to(int64_t pos) {   // everything up to the step's end position
        if (pos == head) {           // ring empty again
            head = tail = used = 0;
            return;
        }
        int64_t freed = pos >= tail ? pos - tail : (cap - tail) + pos;
        tail = pos;
        used -= freed;
        if (used < 0) used = 0;
    }
};

double now_s(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" rtg_status rtg_serve_run(const rtg_scene* scenes, int32_t nscenes, const rtg_request* reqs, int64_t nreq,
                                    const rtg_serve_options* opt, rtg_request_times* times) {
    if (!scenes || nscenes <= 0 || nscenes > kMaxBatchScenes || !reqs || nreq < 0 || !opt || !times) {
        set_last_error("bad serve arguments (1..64 scenes)");
        return RTG_INVALID_PARAM;
    }
    const int dev = scenes[0]->device;
    for (int i = 0; i < nscenes; ++i) {
        if (!scenes[i] || scenes[i]->device != dev || !scenes[i]->built || scenes[i]->hp.ncells == 0) {
            set_last_error("every scene must be built, non-empty and on one device");
            return RTG_INVALID_PARAM;
        }
    }
    const int in_flight = opt->plain ? 1 : std::max(1, std::min(kMaxInFlight, (int)opt->max_in_flight));
    const int64_t max_step_rays = opt->max_step_rays > 0 ? opt->max_step_rays : ((int64_t)1 << 24);
    Ring pool;
    pool.cap = opt->pool_bytes;
    for (int64_t r = 0; r < nreq; ++r) {
        const rtg_request& q = reqs[r];
        const int64_t bytes = align256(32 * q.n) + align256(q.mode == RTG_MODE_ANY ? q.n : 16 * q.n);
        if (q.scene < 0 || q.scene >= nscenes || q.n <= 0 || !q.h_rays || !q.h_out || bytes > pool.cap ||
            (q.mode != RTG_MODE_NEAREST && q.mode != RTG_MODE_ANY) || (r && q.arrival_s < reqs[r - 1].arrival_s)) {
            set_last_error("bad request (scene, size, mode, pool room, or arrivals not sorted)");
            return RTG_INVALID_PARAM;
        }
    }
    if (cudaSetDevice(dev) != cudaSuccess) {
        set_last_error("cudaSetDevice");
        return RTG_DEVICE_ERROR;
    }
    TraceTuning tune = scenes[0]->tune;
    if (opt->empty_run == 2 || opt->empty_run == 4 || opt->empty_run == 8 || opt->empty_run == 16)
        tune.empty_run = opt->empty_run;

    // ---- resources (reserved before the clock starts) -----------------------
    unsigned char* d_pool = nullptr;
    BatchScene* d_scenes = nullptr;
    std::vector<Step> steps(in_flight);
    rtg_status rc = RTG_OK;
    auto cleanup = [&]() {
        cudaDeviceSynchronize();
        for (Step& s : steps) {
            if (s.stream) cudaStreamDestroy(s.stream);
            if (s.done) cudaEventDestroy(s.done);
            if (s.h_tasks) cudaFreeHost(s.h_tasks);
            cudaFree(s.d_tasks);
            cudaFree(s.d_counter);
            cudaFree(s.d_defer);
        }
        cudaFree(d_pool);
        cudaFree(d_scenes);
    };
    if (cudaMalloc(&d_pool, (size_t)pool.cap) != cudaSuccess || cudaMalloc(&d_scenes, sizeof(BatchScene) * nscenes))
        rc = RTG_NO_MEMORY;
    for (Step& s : steps) {
        if (rc) break;
        if (cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming) != cudaSuccess ||
            cudaMallocHost(&s.h_tasks, sizeof(BatchTask) * kMaxStepTasks) != cudaSuccess ||
            cudaMalloc(&s.d_tasks, sizeof(BatchTask) * kMaxStepTasks) != cudaSuccess ||
            cudaMalloc(&s.d_counter, 3 * sizeof(unsigned long long)) != cudaSuccess ||
            cudaMalloc(&s.d_defer, sizeof(int2) * kDeferCap) != cudaSuccess)
            rc = RTG_NO_MEMORY;
    }
    if (rc == RTG_OK) {
        std::vector<BatchScene> hs(nscenes);
        for (int i = 0; i < nscenes; ++i) hs[i].view = scene_view(scenes[i]);
        if (cudaMemcpy(d_scenes, hs.data(), sizeof(BatchScene) * nscenes, cudaMemcpyHostToDevice) != cudaSuccess)
            rc = RTG_DEVICE_ERROR;
        for (int i = 0; i < nscenes && rc == RTG_OK; ++i)
            if (cudaStreamSynchronize(scenes[i]->stream) != cudaSuccess) rc = RTG_DEVICE_ERROR;
    }
    if (rc != RTG_OK) {
        cleanup();
        set_last_error("serve: could not reserve pool, streams or tables");
        return rc;
    }

    // ---- the loop ----------------------------------------------------------
    const auto t0 = std::chrono::steady_clock::now();
    std::deque<int64_t> pending;
    int64_t next = 0, completed = 0;
    int slot_next = 0;                 // steps are launched round-robin over slots
    std::deque<int> order;             // slots in launch order (for in-order release)
    while (completed < nreq) {
        double now = now_s(t0);
        while (next < nreq && reqs[next].arrival_s <= now) pending.push_back(next++);
        // completions (any order), releases (launch order)
        for (int si : order) {
            Step& s = steps[si];
            if (s.busy && !s.reported) {
                cudaError_t q = cudaEventQuery(s.done);
                if (q == cudaSuccess) {
                    const double t = now_s(t0);
                    for (int64_t r : s.reqs) times[r].done_s = t;
                    completed += (int64_t)s.reqs.size();
                    s.reported = true;
                } else if (q != cudaErrorNotReady) {
                    cleanup();
                    set_last_error(std::string("serve step failed: ") + cudaGetErrorString(q));
                    return RTG_DEVICE_ERROR;
                }
            }
        }
        while (!order.empty() && steps[order.front()].reported) {
            Step& s = steps[order.front()];
            pool.release_to(s.pool_end);
            s.busy = false;
            s.reqs.clear();
            order.pop_front();
        }
        // launch a step when a slot is free and requests wait
        Step& s = steps[slot_next];
        if (!pending.empty() && !s.busy) {
            int64_t rays = 0, first = 0;
            int ntasks = 0;
            const double admit = now_s(t0);
            while (!pending.empty() && ntasks < kMaxStepTasks) {
                const rtg_request& q = reqs[pending.front()];
                if (ntasks > 0 && (opt->plain || rays + q.n > max_step_rays)) break;
                const int64_t out_bytes = q.mode == RTG_MODE_ANY ? q.n : 16 * q.n;
                int64_t off_r = 0, off_o = 0;
                const Ring saved = pool;
                if (!pool.alloc(align256(32 * q.n), &off_r)) break;
                if (!pool.alloc(align256(out_bytes), &off_o)) {
                    pool = saved;
                    break;
                }
                const int64_t r = pending.front();
                pending.pop_front();
                times[r].admit_s = admit;
                cudaMemcpyAsync(d_pool + off_r, q.h_rays, 32 * q.n, cudaMemcpyHostToDevice, s.stream);
                BatchTask& T = s.h_tasks[ntasks++];
                T.first = first;
                T.n = q.n;
                T.rays = reinterpret_cast<const float4*>(d_pool + off_r);
                T.out = d_pool + off_o;
                T.scene = q.scene;
                T.mode = q.mode;
                first += (q.n + 31) / 32 * 32;
                rays += q.n;
                s.reqs.push_back(r);
            }
            if (ntasks > 0) {
                if (opt->plain) {
                    // one request through the single-scene kernels
                    const BatchTask& T = s.h_tasks[0];
                    rtg_scene sc = scenes[T.scene];
                    TraceTuning t1 = sc->tune;
                    t1.empty_run = tune.empty_run;
                    if (T.mode == RTG_MODE_ANY)
                        launch_trace_any(scene_view(sc), T.rays, T.n, static_cast<uint8_t*>(T.out), nullptr,
                                         scene_counter(sc), t1, sc->num_sms, s.stream);
                    else
                        launch_trace_nearest(scene_view(sc), T.rays, T.n, static_cast<int4*>(T.out), nullptr,
                                             scene_counter(sc), t1, sc->num_sms, s.stream);
                } else {
                    cudaMemcpyAsync(s.d_tasks, s.h_tasks, sizeof(BatchTask) * ntasks, cudaMemcpyHostToDevice,
                                    s.stream);
                    launch_trace_batch(d_scenes, nscenes, s.d_tasks, ntasks, first,
                                       TraceSlot{s.d_counter, s.d_defer, kDeferCap}, tune, scenes[0]->num_sms,
                                       s.stream);
                }
                for (int t = 0; t < ntasks; ++t) {
                    const rtg_request& q = reqs[s.reqs[t]];
                    const BatchTask& T = s.h_tasks[t];
                    cudaMemcpyAsync(q.h_out, T.out, q.mode == RTG_MODE_ANY ? q.n : 16 * q.n, cudaMemcpyDeviceToHost,
                                    s.stream);
                }
                cudaEventRecord(s.done, s.stream);
                cudaError_t e = cudaGetLastError();
                if (e != cudaSuccess) {
                    cleanup();
                    set_last_error(std::string("serve launch failed: ") + cudaGetErrorString(e));
                    return RTG_DEVICE_ERROR;
                }
                s.pool_end = pool.head;
                s.busy = true;
                s.reported = false;
                order.push_back(slot_next);
                slot_next = (slot_next + 1) % in_flight;
                continue;
            }
        }
        // idle: nothing to launch right now
        if (pending.empty() && next < nreq && order.empty()) {
            const double wait = reqs[next].arrival_s - now_s(t0);
            if (wait > 200e-6) std::this_thread::sleep_for(std::chrono::microseconds((int64_t)((wait - 100e-6) * 1e6)));
        } else {
            std::this_thread::yield();
        }
    }
    cleanup();
    return RTG_OK;
}
