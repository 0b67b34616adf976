// Edge-aware spatial denoiser of the C ABI (dk_denoise_spatial): the
// reference's simpleSpatialDenoiseKernel (Sources/DenrimRendererKit/Resources/
// Shaders/Denoise.metal:39-115), an a-trous pass weighted by normal, depth,
// albedo and colour distance, run `iterations` times with step widths 1, 2, 4
// ... the way SimpleSpatialDenoiser.encode dispatches it
// (Sources/DenrimRendererKit/Denoising/Denoiser.swift:103-160).  It is the
// comparator of the learned denoiser.
#include <algorithm>
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

// Per-image sums behind the learned denoiser's error estimate (two
// independent half-sample renders A and B of an image, their full render F
// and the three denoised images): over the RGB channels of every pixel,
// (dA - dB)^2, (A - B)^2, (F - dF)^2, dF and F.  One grid row per image;
// FP64 partial sums per block, one atomic add per block and term.
constexpr uint32_t kErrTerms = 5;

// The reference's PNG tone curve before 8-bit quantisation
// (PNGWriter.tonemap, Sources/DenrimRendererKit/Image/PNGWriter.swift:182-188):
// exposure 0.8, the ACES fit, clamp to [0, 1], gamma 1/2.2.
__device__ __forceinline__ float displayValue(float v) {
    const float x = fmaxf(v, 0.0f) * 0.8f;
    const float m = (x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f);
    return powf(fminf(fmaxf(m, 0.0f), 1.0f), 1.0f / 2.2f);
}

__device__ __forceinline__ float4 inDomain(float4 v, uint32_t display) {
    if (!display) return v;
    return make_float4(displayValue(v.x), displayValue(v.y), displayValue(v.z), v.w);
}

__global__ void __launch_bounds__(256) k_error_terms(const float4* __restrict__ a, const float4* __restrict__ b,
                                                     const float4* __restrict__ f, const float4* __restrict__ da,
                                                     const float4* __restrict__ db, const float4* __restrict__ df,
                                                     uint32_t pixels, uint32_t display, double* __restrict__ terms) {
    const size_t base = (size_t)blockIdx.y * pixels;
    double acc[kErrTerms] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < pixels; i += gridDim.x * blockDim.x) {
        const size_t k = base + i;
        const float4 va = inDomain(a[k], display), vb = inDomain(b[k], display), vf = inDomain(f[k], display);
        const float4 vda = inDomain(da[k], display), vdb = inDomain(db[k], display), vdf = inDomain(df[k], display);
        const double dd[3] = {(double)vda.x - vdb.x, (double)vda.y - vdb.y, (double)vda.z - vdb.z};
        const double nn[3] = {(double)va.x - vb.x, (double)va.y - vb.y, (double)va.z - vb.z};
        const double fd[3] = {(double)vf.x - vdf.x, (double)vf.y - vdf.y, (double)vf.z - vdf.z};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            acc[0] += dd[c] * dd[c];
            acc[1] += nn[c] * nn[c];
            acc[2] += fd[c] * fd[c];
        }
        acc[3] += (double)vdf.x + vdf.y + vdf.z;
        acc[4] += (double)vf.x + vf.y + vf.z;
    }
    __shared__ double part[kErrTerms][8];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
    for (uint32_t t = 0; t < kErrTerms; ++t) {
        double v = acc[t];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) part[t][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < kErrTerms) {
        double v = 0.0;
        for (uint32_t w = 0; w < blockDim.x / 32u; ++w) v += part[threadIdx.x][w];
        atomicAdd(terms + (size_t)blockIdx.y * kErrTerms + threadIdx.x, v);
    }
}

// out = (1 - t) a + t b per RGBA texel: the full render of two independent
// renders of n_a and n_b samples with t = n_b / (n_a + n_b) (0.5 for two
// halves; the previous full render and a render of more samples when a
// progressive render grows).
__global__ void __launch_bounds__(256) k_average_planes(const float4* a, const float4* b, float4* out, size_t n, float t) {
    const float s = 1.0f - t;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float4 x = a[i], y = b[i];
        out[i] = make_float4(s * x.x + t * y.x, s * x.y + t * y.y, s * x.z + t * y.z, s * x.w + t * y.w);
    }
}

}  // namespace

}  // namespace dk

extern "C" int dk_average_planes(const float* a, const float* b, float* out, size_t texels, float t, void* stream) {
    if (!a || !b || !out) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_average_planes: null argument");
    if (!(t >= 0.0f && t <= 1.0f)) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_average_planes: t outside [0, 1]");
    if (texels == 0) return DK_OK;
    const unsigned grid = (unsigned)std::min<size_t>((texels + 255u) / 256u, 152u * 16u);
    dk::k_average_planes<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const float4*>(a), reinterpret_cast<const float4*>(b), reinterpret_cast<float4*>(out), texels,
        t);
    DK_CUDA(cudaGetLastError(), "average planes launch");
    return DK_OK;
}

extern "C" int dk_denoise_error_terms(const float* half_a, const float* half_b, const float* full,
                                      const float* denoised_a, const float* denoised_b, const float* denoised_full,
                                      uint32_t pixels, uint32_t images, uint32_t display, double* terms,
                                      void* stream) {
    if (!half_a || !half_b || !full || !denoised_a || !denoised_b || !denoised_full || !terms)
        return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_denoise_error_terms: null argument");
    if (images > 65535u) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "dk_denoise_error_terms: at most 65535 images");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DK_CUDA(cudaMemsetAsync(terms, 0, (size_t)images * dk::kErrTerms * sizeof(double), st), "error terms clear");
    if (pixels == 0 || images == 0) return DK_OK;
    const uint32_t blocks = std::min<uint32_t>((pixels + 255u) / 256u, 64u);
    dk::k_error_terms<<<dim3(blocks, images), 256, 0, st>>>(
        reinterpret_cast<const float4*>(half_a), reinterpret_cast<const float4*>(half_b),
        reinterpret_cast<const float4*>(full), reinterpret_cast<const float4*>(denoised_a),
        reinterpret_cast<const float4*>(denoised_b), reinterpret_cast<const float4*>(denoised_full), pixels,
        display ? 1u : 0u, terms);
    DK_CUDA(cudaGetLastError(), "error terms launch");
    return DK_OK;
}

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
