// trace_any.cu -- the tracer's launches for any-hit of rays given as arrays (MODE_ANY).
// The kernels and their launch helpers live in trace_device.cuh; each mode
// is its own translation unit so the library's kernels compile in parallel.
#include "trace_device.cuh"

namespace gridrt {

void launch_trace_any(const SceneView& s, const float4* rays, int64_t n, uint8_t* occ, TraceCounters* ctr,
                      const TraceSlot& slot, const TraceTuning& tune, int num_sms, cudaStream_t st) {
    if (n <= 0) return;
    TraceIO io{};
    io.rays = rays;
    io.occ = occ;
    io.n = n;
    io.ctr = ctr;
    launch_mode<MODE_ANY>(s, io, slot, tune, num_sms, st);
}

}  // namespace gridrt
