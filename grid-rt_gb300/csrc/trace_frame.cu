// trace_frame.cu -- the tracer's launches for camera rays and, in the same lanes, their shadow rays (MODE_FRAME).
// The kernels and their launch helpers live in trace_device.cuh; each mode
// is its own translation unit so the library's kernels compile in parallel.
#include "trace_device.cuh"

namespace gridrt {

void launch_trace_frame(const SceneView& s, const CameraArgs& cam, int4* hits, const float* light,
                        float4* shadow_rays, uint8_t* occ, TraceCounters* ctr, const TraceSlot& slot,
                        const TraceTuning& tune, int num_sms, cudaStream_t st) {
    const int64_t n = (int64_t)cam.width * cam.height;
    if (n <= 0) return;
    TraceIO io{};
    io.rays = shadow_rays;   // the deferred passes load shadow rays from their slots
    io.hits = hits;
    io.occ = occ;
    io.shadow_rays = shadow_rays;
    io.cam = cam;
    io.light = make_float3(light[0], light[1], light[2]);
    io.has_light = 1;
    io.n = n;
    io.ctr = ctr;
    launch_mode<MODE_FRAME>(s, io, slot, tune, num_sms, st);
}

}  // namespace gridrt
