// probe.cu -- read-bandwidth probe for the roofline denominators.
//
// The traversal's reads are served by L2 when the scene fits in it; the L2
// figure the benchmark divides by is measured here: every thread streams
// 16-byte loads that skip L1 (ld.global.cg) over a buffer of the given size,
// repeatedly, and the kernel's event-timed duration gives bytes / s.  A
// buffer well below the L2 size measures L2, one far above it measures HBM.
#include <string>

#include "../../include/gridrt.h"
#include "kernels.h"

namespace {

__global__ void read_probe_kernel(const float4* __restrict__ p, int64_t n, int reps, float* out) {
    float acc = 0.0f;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int r = 0; r < reps; ++r) {
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const float4 v = __ldcg(p + i);
            acc += (v.x + v.y) + (v.z + v.w);
        }
    }
    if (acc == -1.0f) out[0] = acc;   // never true for the zero-filled buffer; keeps the loads
}

}  // namespace

extern "C" rtg_status rtg_probe_read_gbs(int32_t device, int64_t bytes, int32_t reps, double* gbs) {
    if (!gbs || bytes < 16 || reps <= 0) {
        gridrt::set_last_error("probe: bad arguments");
        return RTG_INVALID_PARAM;
    }
    *gbs = 0.0;
    if (cudaSetDevice(device) != cudaSuccess) {
        gridrt::set_last_error("probe: cudaSetDevice");
        return RTG_DEVICE_ERROR;
    }
    const int64_t n = bytes / 16;
    float4* buf = nullptr;
    float* out = nullptr;
    if (cudaMalloc(&buf, (size_t)n * 16) != cudaSuccess || cudaMalloc(&out, sizeof(float)) != cudaSuccess) {
        cudaFree(buf);
        gridrt::set_last_error("probe: allocation");
        return RTG_NO_MEMORY;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMemset(buf, 0, (size_t)n * 16);
    const int blocks = 8 * (sms > 0 ? sms : 1);
    read_probe_kernel<<<blocks, 256>>>(buf, n, 1, out);   // warm-up (and L2 fill for small buffers)
    float best = 1e30f;
    for (int t = 0; t < 5; ++t) {
        cudaEventRecord(e0);
        read_probe_kernel<<<blocks, 256>>>(buf, n, reps, out);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    cudaFree(out);
    if (err != cudaSuccess) {
        gridrt::set_last_error(std::string("probe: ") + cudaGetErrorString(err));
        return RTG_DEVICE_ERROR;
    }
    *gbs = (double)n * 16.0 * reps / (best * 1e-3) / 1e9;
    return RTG_OK;
}
