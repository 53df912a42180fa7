// trace_camera.cu -- the tracer's launches for camera rays, closest hit, with optional shadow or diffuse secondary rays (MODE_CAMERA).
// The kernels and their launch helpers live in trace_device.cuh; each mode
// is its own translation unit so the library's kernels compile in parallel.
#include "trace_device.cuh"

namespace gridrt {

void launch_trace_camera(const SceneView& s, const CameraArgs& cam, int4* hits, const float* light,
                         float4* shadow_rays, TraceCounters* ctr, const TraceSlot& slot,
                         const TraceTuning& tune, int num_sms, cudaStream_t st, int diffuse,
                         unsigned long long seed) {
    const int64_t n = (int64_t)cam.width * cam.height;
    if (n <= 0) return;
    TraceIO io{};
    io.diffuse = diffuse;
    io.seed = seed;
    io.hits = hits;
    io.shadow_rays = shadow_rays;
    io.cam = cam;
    io.light = light ? make_float3(light[0], light[1], light[2]) : make_float3(0.f, 0.f, 0.f);
    io.has_light = light != nullptr;
    io.n = n;
    io.ctr = ctr;
    launch_mode<MODE_CAMERA>(s, io, slot, tune, num_sms, st);
}

}  // namespace gridrt
