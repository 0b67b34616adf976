// Edge-aware spatial denoiser of the C ABI (dk_denoise_spatial): the
// reference's simpleSpatialDenoiseKernel (Sources/DenrimRendererKit/Resources/
// Shaders/Denoise.metal:39-115), an a-trous pass weighted by normal, depth,
// albedo and colour distance, run `iterations` times with step widths 1, 2, 4
// ... the way SimpleSpatialDenoiser.encode dispatches it
// (Sources/DenrimRendererKit/Denoising/Denoiser.swift:103-160).  It is the
// comparator of the learned denoiser.
#include <cstdint>

#include "dk_host.h"

namespace dk {

namespace {

__device__ __forceinline__ float3 denoiseNormal(float4 e) {
    float3 v = make_float3(e.x * 2.0f - 1.0f, e.y * 2.0f - 1.0f, e.z * 2.0f - 1.0f);
    float inv = 1.0f / sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    return make_float3(v.x * inv, v.y * inv, v.z * inv);
}

__device__ __forceinline__ float colorDistance(float3 a, float3 b) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return dx * dx + dy * dy + dz * dz;
}

__device__ __forceinline__ float kernelWeight(int offset) {
    int a = offset < 0 ? -offset : offset;
    return a == 0 ? 0.375f : (a == 1 ? 0.25f : 0.0625f);
}

struct SpatialParams {
    uint32_t width, height, radius, stepWidth;
    float normalSigma, depthSigma, albedoSigma, colorSigma;
};

__global__ void __launch_bounds__(256) k_spatial_denoise(const float4* __restrict__ beauty,
                                                         const float4* __restrict__ depth,
                                                         const float4* __restrict__ normal,
                                                         const float4* __restrict__ albedo, float4* __restrict__ out,
                                                         SpatialParams c) {
    uint32_t gx = blockIdx.x * 16 + threadIdx.x % 16, gy = blockIdx.y * 16 + threadIdx.x / 16;
    if (gx >= c.width || gy >= c.height) return;
    size_t idx = (size_t)gy * c.width + gx;
    float4 cb = beauty[idx];
    float cd = depth[idx].x;
    if (cb.w <= 0.0001f || !isfinite(cd) || cd <= 0.0f) {
        out[idx] = cb;
        return;
    }
    float3 cn = denoiseNormal(normal[idx]);
    float4 ca4 = albedo[idx];
    float3 ca = make_float3(ca4.x, ca4.y, ca4.z);
    float3 cc = make_float3(cb.x, cb.y, cb.z);
    int radius = (int)c.radius;
    float nS2 = c.normalSigma * c.normalSigma;
    float dS = fmaxf(c.depthSigma * fmaxf(cd, 1.0f), 0.0001f);
    float dS2 = dS * dS;
    float aS2 = c.albedoSigma * c.albedoSigma;
    float cS2 = c.colorSigma * c.colorSigma;
    int step = (int)(c.stepWidth > 1u ? c.stepWidth : 1u);
    float3 acc = make_float3(0.0f, 0.0f, 0.0f);
    float total = 0.0f;
    for (int y = -radius; y <= radius; ++y) {
        for (int x = -radius; x <= radius; ++x) {
            int sx = min(max((int)gx + x * step, 0), (int)c.width - 1);
            int sy = min(max((int)gy + y * step, 0), (int)c.height - 1);
            size_t s = (size_t)sy * c.width + sx;
            float4 sb = beauty[s];
            float sd = depth[s].x;
            if (sb.w <= 0.0001f || !isfinite(sd) || sd <= 0.0f) continue;
            float spatial = kernelWeight(x) * kernelWeight(y);
            float3 sn = denoiseNormal(normal[s]);
            float nd = 1.0f - fminf(fmaxf(cn.x * sn.x + cn.y * sn.y + cn.z * sn.z, 0.0f), 1.0f);
            float nw = expf(-(nd * nd) / (2.0f * nS2));
            float dd = sd - cd;
            float dw = expf(-(dd * dd) / (2.0f * dS2));
            float4 sa4 = albedo[s];
            float aw = expf(-colorDistance(ca, make_float3(sa4.x, sa4.y, sa4.z)) / (2.0f * aS2));
            float cw = expf(-colorDistance(cc, make_float3(sb.x, sb.y, sb.z)) / (2.0f * cS2));
            float w = spatial * nw * dw * aw * cw;
            acc.x += sb.x * w;
            acc.y += sb.y * w;
            acc.z += sb.z * w;
            total += w;
        }
    }
    float3 d = total > 0.0f ? make_float3(acc.x / total, acc.y / total, acc.z / total) : cc;
    // mix(center, denoised, 0.85)
    out[idx] = make_float4(cc.x + (d.x - cc.x) * 0.85f, cc.y + (d.y - cc.y) * 0.85f, cc.z + (d.z - cc.z) * 0.85f, cb.w);
}

}  // namespace

}  // namespace dk

extern "C" int dk_denoise_spatial(const float* beauty, const float* depth, const float* normal, const float* albedo,
                                  float* out, float* scratch, uint32_t width, uint32_t height,
                                  const dk_spatial_denoise_settings* settings, void* stream) {
    if (!beauty || !depth || !normal || !albedo || !out || !settings || (settings->iterations > 1 && !scratch))
        return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_denoise_spatial: null argument");
    if (width == 0 || height == 0) return DK_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    dk::SpatialParams c;
    c.width = width;
    c.height = height;
    c.radius = settings->radius < 1 ? 1 : (settings->radius > 2 ? 2 : settings->radius);
    c.normalSigma = fmaxf(settings->normal_sigma, 0.0001f);
    c.depthSigma = fmaxf(settings->depth_sigma, 0.0001f);
    c.albedoSigma = fmaxf(settings->albedo_sigma, 0.0001f);
    c.colorSigma = fmaxf(settings->color_sigma, 0.0001f);
    uint32_t iterations = settings->iterations < 1 ? 1 : (settings->iterations > 5 ? 5 : settings->iterations);
    const size_t plane = (size_t)width * height;
    const float4* src = reinterpret_cast<const float4*>(beauty);
    float4* tmp[2] = {reinterpret_cast<float4*>(scratch), reinterpret_cast<float4*>(scratch) + plane};
    dim3 grid((width + 15) / 16, (height + 15) / 16);
    for (uint32_t it = 0; it < iterations; ++it) {
        float4* dst = it == iterations - 1 ? reinterpret_cast<float4*>(out) : tmp[it & 1u];
        c.stepWidth = 1u << it;
        dk::k_spatial_denoise<<<grid, 256, 0, st>>>(src, reinterpret_cast<const float4*>(depth),
                                                    reinterpret_cast<const float4*>(normal),
                                                    reinterpret_cast<const float4*>(albedo), dst, c);
        src = dst;
    }
    DK_CUDA(cudaGetLastError(), "spatial denoise launch");
    return DK_OK;
}
