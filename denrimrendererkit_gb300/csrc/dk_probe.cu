// Bandwidth probe of the C ABI (dk_probe_bandwidth): the measured L2 and HBM
// read bandwidths that the traversal stages' rooflines are stated against.
// A read-only sweep with 16-byte loads over a buffer: one that fits in L2
// (the sweep is then served by L2 after its first pass) or one far larger
// (served by HBM).  Persistent CTAs, `passes` sweeps per launch, timed with
// CUDA events on the caller's stream.  Measurement only; no counterpart in
// the reference.
#include <algorithm>
#include <cstdint>

#include "dk_host.h"

namespace dk {
namespace {

__global__ void __launch_bounds__(512) k_probe_read(const float4* __restrict__ buf, size_t n4, uint32_t passes,
                                                    float* __restrict__ sink) {
    float acc = 0.0f;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (uint32_t p = 0; p < passes; ++p) {
        // Each pass starts at another offset so no CTA re-reads its own lines.
        const size_t shift = ((size_t)p * 4099u * blockDim.x) % n4;
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += stride) {
            size_t j = i + shift;
            if (j >= n4) j -= n4;
            const float4 v = __ldcg(buf + j);
            acc += v.x + v.y + v.z + v.w;
        }
    }
    if (acc == 12345.678f) sink[0] = acc;  // keeps the loads
}

}  // namespace
}  // namespace dk

extern "C" int dk_probe_bandwidth(uint64_t bytes, uint32_t passes, double* out_gbs, void* stream) {
    if (!out_gbs || bytes < (1u << 20) || passes == 0)
        return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_probe_bandwidth: at least 1 MiB and one pass");
    int rc = dk::ensureDevice();
    if (rc != DK_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t n4 = bytes / sizeof(float4);
    float4* buf = nullptr;
    float* sink = nullptr;
    DK_CUDA(cudaMalloc(&buf, n4 * sizeof(float4)), "probe buffer");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&] {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        cudaFree(buf);
        if (sink) cudaFree(sink);
    };
    cudaError_t e = cudaMemsetAsync(buf, 0, n4 * sizeof(float4), st);
    if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(float));
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    const int sms = dk::deviceProp().multiProcessorCount > 0 ? dk::deviceProp().multiProcessorCount : 1;
    const int grid = sms * 4;
    if (e == cudaSuccess) {
        dk::k_probe_read<<<grid, 512, 0, st>>>(buf, n4, 1, sink);  // warm-up (and fills L2 for a small buffer)
        e = cudaEventRecord(e0, st);
    }
    if (e == cudaSuccess) {
        dk::k_probe_read<<<grid, 512, 0, st>>>(buf, n4, passes, sink);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cleanup();
    if (e != cudaSuccess) return dk::fail(DK_ERROR_COMMAND_FAILED, std::string("bandwidth probe: ") + cudaGetErrorString(e));
    *out_gbs = (double)n4 * sizeof(float4) * passes / (ms * 1e-3) / 1e9;
    return DK_OK;
}
