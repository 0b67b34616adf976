// Allocation-free variant of the environment importance-table builder.
//
// dk_build_environment_samples() copies a host image to the device and
// allocates its FP64 working memory with cudaMalloc on every call.  Some
// callers cannot do that: a host application that hands the renderer only
// memory from its own device arena or pool (and forbids the library from
// allocating behind its back), or a real-time frame loop that must not pay for
// — or stall on — a device allocation.  dk_build_environment_samples_noalloc()
// serves them: the caller passes device pointers for the input texels and the
// output table, and the FP64 prefix-sum scratch lives in one file-scope
// `static __device__` array of a fixed maximum size, which every GPU that loads
// this library holds until the process exits.
//
// The arithmetic is the same as the allocating builder's (FP64 weights and
// prefix sum, FP32 results), so both produce the same table.
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/denrim_cuda.h"

namespace dk {
void setLastError(const std::string& message);  // dk_host.cu: the dk_last_error_message() slot
}

namespace {

constexpr uint32_t kMaxTexels = DK_ENV_NOALLOC_MAX_TEXELS;
constexpr uint32_t kBlock = 1024u;
constexpr uint32_t kMaxBlocks = (kMaxTexels + kBlock - 1u) / kBlock;

// [0, kMaxTexels): FP64 weights, scanned in place into per-block prefixes;
// [kMaxTexels, kMaxTexels + kMaxBlocks]: block offsets, then the total.
static __device__ __align__(256) double g_envScratch[kMaxTexels + kMaxBlocks + 64];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_scratchPtr[kMaxDevices] = {};

__device__ __forceinline__ double texelWeight(const float4* px, uint32_t i, uint32_t w, uint32_t h, float intensity,
                                              float maxR) {
    double dTheta = 3.141592653589793 / (double)h, dPhi = 2.0 * 3.141592653589793 / (double)w;
    uint32_t y = i / w;
    double theta = ((double)y + 0.5) * dTheta;
    double solid = fmax(sin(theta) * dTheta * dPhi, 1e-8);
    float4 t = px[i];
    double r = (double)t.x * intensity, g = (double)t.y * intensity, b = (double)t.z * intensity;
    if (maxR > 0.0f) {
        r = fmin(r, (double)maxR);
        g = fmin(g, (double)maxR);
        b = fmin(b, (double)maxR);
    }
    double lum = r * 0.2126 + g * 0.7152 + b * 0.0722;
    return fmax(lum, 0.0) * solid;
}

__global__ void k_na_weights(const float4* px, uint32_t w, uint32_t h, float intensity, float maxR, double* s) {
    uint32_t n = w * h;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        s[i] = texelWeight(px, i, w, h, intensity, maxR);
}

__global__ void __launch_bounds__(1024) k_na_scan_block(double* data, uint32_t n, double* blockSums) {
    __shared__ double warpSums[32];
    uint32_t lane = threadIdx.x & 31u;
    uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    double v = i < n ? data[i] : 0.0;
    for (int o = 1; o < 32; o <<= 1) {
        double u = __shfl_up_sync(0xffffffffu, v, o);
        if ((int)lane >= o) v += u;
    }
    if (lane == 31u) warpSums[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32u) {
        double ws = warpSums[threadIdx.x];
        for (int o = 1; o < 32; o <<= 1) {
            double u = __shfl_up_sync(0xffffffffu, ws, o);
            if ((int)threadIdx.x >= o) ws += u;
        }
        warpSums[threadIdx.x] = ws;
    }
    __syncthreads();
    if ((threadIdx.x >> 5) > 0u) v += warpSums[(threadIdx.x >> 5) - 1u];
    if (i < n) data[i] = v;
    if (threadIdx.x == kBlock - 1u) blockSums[blockIdx.x] = v;
}

__global__ void k_na_scan_totals(double* blockSums, uint32_t nb) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double acc = 0.0;
    for (uint32_t b = 0; b < nb; ++b) {
        double t = blockSums[b];
        blockSums[b] = acc;
        acc += t;
    }
    blockSums[nb] = acc;
}

__global__ void k_na_finish(const float4* px, uint32_t w, uint32_t h, float intensity, float maxR, const double* prefix,
                            const double* blockSums, uint32_t nb, float2* out) {
    uint32_t n = w * h;
    double total = blockSums[nb];
    double dTheta = 3.141592653589793 / (double)h, dPhi = 2.0 * 3.141592653589793 / (double)w;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double cum = prefix[i] + blockSums[i / kBlock];
        uint32_t y = i / w;
        double theta = ((double)y + 0.5) * dTheta;
        double solid = fmax(sin(theta) * dTheta * dPhi, 1e-8);
        double prob = texelWeight(px, i, w, h, intensity, maxR) / total;
        out[i] = make_float2((float)fmin(cum / total, 1.0), (float)(prob / solid));
    }
}

int naFail(int code, const char* msg, cudaError_t e = cudaSuccess) {
    std::string m = msg;
    if (e != cudaSuccess) {
        m += ": ";
        m += cudaGetErrorString(e);
    }
    dk::setLastError(m);
    return code;
}

// Device address of the static scratch on the current device, looked up once
// per device (the host-side name of a __device__ array is not its address).
int scratchForCurrentDevice(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return naFail(DK_ERROR_NO_DEVICE, "dk_build_environment_samples_noalloc: no current device", e);
    if (dev < 0 || dev >= kMaxDevices) return naFail(DK_ERROR_INVALID_ARGUMENT, "device ordinal too large");
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratchPtr[dev]) {
        double* ptr = nullptr;
        e = cudaGetSymbolAddress((void**)&ptr, g_envScratch);
        if (e != cudaSuccess || !ptr)
            return naFail(DK_ERROR_COMMAND_FAILED, "cudaGetSymbolAddress of the static scratch failed", e);
        g_scratchPtr[dev] = ptr;
    }
    *out = g_scratchPtr[dev];
    return DK_OK;
}

}  // namespace

extern "C" {

int dk_build_environment_samples_noalloc(const dk_float4* device_pixels, uint32_t width, uint32_t height,
                                         float intensity, float max_radiance, dk_environment_sample* device_out,
                                         uint32_t* out_count, void* stream) {
    if (!out_count) return naFail(DK_ERROR_INVALID_ARGUMENT, "out_count is null");
    *out_count = 0;
    if (width == 0 || height == 0) return DK_OK;
    if (!device_pixels || !device_out) return naFail(DK_ERROR_INVALID_ARGUMENT, "device_pixels or device_out is null");
    // The kernels read float4 texels and write float2 entries: both pointers
    // must be aligned for those and must be device (or managed) memory, so a
    // host or misaligned pointer is an error here, not a fault in the context.
    if (reinterpret_cast<uintptr_t>(device_pixels) % 16u != 0 || reinterpret_cast<uintptr_t>(device_out) % 8u != 0)
        return naFail(DK_ERROR_INVALID_ARGUMENT,
                      "dk_build_environment_samples_noalloc: device_pixels must be 16-byte and device_out 8-byte "
                      "aligned");
    for (const void* ptr : {static_cast<const void*>(device_pixels), static_cast<const void*>(device_out)}) {
        cudaPointerAttributes attr{};
        cudaError_t pe = cudaPointerGetAttributes(&attr, ptr);
        if (pe != cudaSuccess) {
            cudaGetLastError();
            return naFail(DK_ERROR_INVALID_ARGUMENT, "dk_build_environment_samples_noalloc: unknown pointer", pe);
        }
        if (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)
            return naFail(DK_ERROR_INVALID_ARGUMENT,
                          "dk_build_environment_samples_noalloc: device_pixels and device_out must be device memory");
    }
    uint64_t n64 = (uint64_t)width * height;
    if (n64 > kMaxTexels)
        return naFail(DK_ERROR_INVALID_ARGUMENT,
                      "dk_build_environment_samples_noalloc: map exceeds the static scratch maximum of "
                      "DK_ENV_NOALLOC_MAX_TEXELS (2048 x 1024) texels; use dk_build_environment_samples");
    uint32_t n = (uint32_t)n64;
    double* scratch = nullptr;
    int rc = scratchForCurrentDevice(&scratch);
    if (rc != DK_OK) return rc;
    double* blockSums = scratch + kMaxTexels;
    uint32_t nb = (n + kBlock - 1u) / kBlock;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // The call reads the table's total back to the host and waits for it,
    // which a stream under capture cannot do: such a call is refused.
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    cudaError_t ce = cudaStreamIsCapturing(st, &capture);
    if (ce != cudaSuccess || capture != cudaStreamCaptureStatusNone) {
        if (ce != cudaSuccess) cudaGetLastError();
        return naFail(DK_ERROR_INVALID_ARGUMENT,
                      "dk_build_environment_samples_noalloc: the stream is being captured (or invalid)", ce);
    }
    // An error left by unrelated earlier work is not this call's failure.
    cudaGetLastError();
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int grid = 4 * (sms > 0 ? sms : 1);
    const float4* px = reinterpret_cast<const float4*>(device_pixels);
    float I = intensity > 0.0f ? intensity : 0.0f;
    float M = max_radiance > 0.0f ? max_radiance : 0.0f;
    // Every call overwrites the scratch it reads; the block offsets and the
    // total start from zero so nothing of the previous call leaks in.
    cudaError_t e = cudaMemsetAsync(blockSums, 0, sizeof(double) * (nb + 1u), st);
    if (e != cudaSuccess) return naFail(DK_ERROR_COMMAND_FAILED, "clearing the scratch failed", e);
    k_na_weights<<<grid, 256, 0, st>>>(px, width, height, I, M, scratch);
    k_na_scan_block<<<nb, kBlock, 0, st>>>(scratch, n, blockSums);
    k_na_scan_totals<<<1, 32, 0, st>>>(blockSums, nb);
    e = cudaGetLastError();
    if (e != cudaSuccess) return naFail(DK_ERROR_COMMAND_FAILED, "environment table (no-alloc) launch failed", e);
    double total = 0.0;
    e = cudaMemcpyAsync(&total, blockSums + nb, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return naFail(DK_ERROR_COMMAND_FAILED, "environment table (no-alloc) failed", e);
    if (!(total > 0.0)) return DK_OK;  // no energy: the reference's empty table
    k_na_finish<<<grid, 256, 0, st>>>(px, width, height, I, M, scratch, blockSums, nb,
                                      reinterpret_cast<float2*>(device_out));
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return naFail(DK_ERROR_COMMAND_FAILED, "environment table (no-alloc) failed", e);
    *out_count = n;
    return DK_OK;
}

}  // extern "C"
