// Spatiotemporal variance-guided filtering (SVGF) of the C ABI (dk_svgf_*):
// the temporal denoiser the reference selects as DenoiseSettings.appleSVGF
// (Sources/DenrimRendererKit/Denoising/Denoiser.swift:67-76, 167-300).  The
// reference drives Apple's closed MPSSVGFDenoiser; this is the published
// algorithm (Schied et al., "Spatiotemporal Variance-Guided Filtering",
// HPG 2017) with the parameters the reference's configure(settings:) sets
// (Denoiser.swift:227-237) and the edge-stopping functions Apple documents
// for them:
//   depth     exp(-|z_p - z_q| / depthWeight)
//   normal    max(0, n_p . n_q) ^ normalWeight
//   luminance exp(-|l_p - l_q| / (luminanceWeight * sigma_l(p) + eps))
// where sigma_l is the standard deviation from the 3x3-prefiltered variance.
//
// Per frame: pack depth + signed normal (the reference's
// packSVGFDepthNormalKernel, Denoise.metal:117-136, exact operations);
// reproject the previous frame's integrated colour and luminance moments
// through the motion-vector AOV (previous pixel = pixel + motion,
// PathTrace.metal:5569-5577) with depth/normal consistency tests and blend
// them by an exponential moving average (factor 0.2, at least 1/history);
// estimate the variance from the temporal moments, or spatially over the
// variance-estimation radius while the history is shorter than 4 frames;
// then `iterations` a-trous passes (step 1, 2, 4, ...), the first pass's
// result feeding the next frame's history; finally the reference's
// copySVGFOutputKernel (Denoise.metal:138-154, exact operations).
#include <algorithm>
#include <cstdint>

#include "dk_host.h"

namespace dk {

namespace {

constexpr float kInvalidDepth = 1.0e6f;
constexpr float kHistoryCap = 32.0f;
constexpr float kReprojectDepth = 0.1f;   // relative depth difference accepted by reprojection
constexpr float kReprojectNormal = 0.9f;  // cosine accepted by reprojection

struct SvgfParams {
    uint32_t width, height;
    int radius, varianceRadius, step;
    float depthWeight, normalWeight, luminanceWeight;
    float bilateralSigma, varianceSigma, prefilterSigma;
    float alpha, alphaMoments;
    int hasHistory, writeHistory;
};

__device__ __forceinline__ float luminance(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

__device__ __forceinline__ bool inside(int x, int y, const SvgfParams& p) {
    return x >= 0 && y >= 0 && x < (int)p.width && y < (int)p.height;
}

// packSVGFDepthNormalKernel: (depth, normalize(encoded * 2 - 1)); pixels
// without a surface get (1e6, 0, 0, 1).
__global__ void __launch_bounds__(256) k_svgf_pack(const float4* __restrict__ depth, const float4* __restrict__ normal,
                                                   float4* __restrict__ out, uint32_t width, uint32_t height) {
    uint32_t x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
    if (x >= width || y >= height) return;
    size_t i = (size_t)y * width + x;
    float4 d = depth[i], e = normal[i];
    if (e.w <= 0.0001f || !isfinite(d.x) || d.x <= 0.0f) {
        out[i] = make_float4(kInvalidDepth, 0.0f, 0.0f, 1.0f);
        return;
    }
    float vx = __fsub_rn(__fmul_rn(e.x, 2.0f), 1.0f);
    float vy = __fsub_rn(__fmul_rn(e.y, 2.0f), 1.0f);
    float vz = __fsub_rn(__fmul_rn(e.z, 2.0f), 1.0f);
    float dd = __fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz));
    float inv = __fdiv_rn(1.0f, __fsqrt_rn(dd));
    out[i] = make_float4(d.x, __fmul_rn(vx, inv), __fmul_rn(vy, inv), __fmul_rn(vz, inv));
}

// Temporal reprojection + moving average.  Writes the integrated colour to
// `integrated` (rgb) and the moments (mu1, mu2, history length) to `moments`.
__global__ void __launch_bounds__(256) k_svgf_temporal(const float4* __restrict__ beauty,
                                                       const float4* __restrict__ motion,
                                                       const float4* __restrict__ dnCur,
                                                       const float4* __restrict__ dnPrev,
                                                       const float4* __restrict__ histColor,
                                                       const float4* __restrict__ histMoments,
                                                       float4* __restrict__ integrated, float4* __restrict__ moments,
                                                       SvgfParams p) {
    int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
    if (x >= (int)p.width || y >= (int)p.height) return;
    size_t i = (size_t)y * p.width + x;
    float4 b = beauty[i];
    float3 c = make_float3(b.x, b.y, b.z);
    float l = luminance(c);
    float4 dn = dnCur[i];
    float3 sumC = make_float3(0.0f, 0.0f, 0.0f);
    float sumM1 = 0.0f, sumM2 = 0.0f, sumLen = 0.0f, sumW = 0.0f;
    float4 mv = motion[i];
    if (p.hasHistory && mv.w > 0.0f && dn.x < kInvalidDepth) {
        // previous-frame pixel coordinates of this pixel's surface point
        float px = (float)x + mv.x, py = (float)y + mv.y;
        float fx0 = floorf(px), fy0 = floorf(py);
        float fx = px - fx0, fy = py - fy0;
        int x0 = (int)fx0, y0 = (int)fy0;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            int qx = x0 + (t & 1), qy = y0 + (t >> 1);
            float w = ((t & 1) ? fx : 1.0f - fx) * ((t >> 1) ? fy : 1.0f - fy);
            if (w <= 0.0f || !inside(qx, qy, p)) continue;
            size_t j = (size_t)qy * p.width + qx;
            float4 dq = dnPrev[j];
            if (dq.x >= kInvalidDepth) continue;
            if (fabsf(dq.x - dn.x) > kReprojectDepth * fmaxf(dn.x, 1.0e-3f)) continue;
            if (dq.y * dn.y + dq.z * dn.z + dq.w * dn.w < kReprojectNormal) continue;
            float4 hc = histColor[j], hm = histMoments[j];
            sumC.x += w * hc.x;
            sumC.y += w * hc.y;
            sumC.z += w * hc.z;
            sumM1 += w * hm.x;
            sumM2 += w * hm.y;
            sumLen += w * hm.z;
            sumW += w;
        }
    }
    float4 outC, outM;
    if (sumW > 1.0e-4f) {
        float inv = 1.0f / sumW;
        float len = fminf(sumLen * inv + 1.0f, kHistoryCap);
        float a = fmaxf(p.alpha, 1.0f / len), am = fmaxf(p.alphaMoments, 1.0f / len);
        float3 hc = make_float3(sumC.x * inv, sumC.y * inv, sumC.z * inv);
        outC = make_float4(hc.x + (c.x - hc.x) * a, hc.y + (c.y - hc.y) * a, hc.z + (c.z - hc.z) * a, 0.0f);
        float m1 = sumM1 * inv, m2 = sumM2 * inv;
        outM = make_float4(m1 + (l - m1) * am, m2 + (l * l - m2) * am, len, 0.0f);
    } else {
        outC = make_float4(c.x, c.y, c.z, 0.0f);
        outM = make_float4(l, l * l, 1.0f, 0.0f);
    }
    integrated[i] = outC;
    moments[i] = outM;
}

// Variance: from the temporal moments once 4 frames are integrated, else a
// bilateral estimate over the variance-estimation radius (boosted by 4 / n
// for young histories).  Output (rgb, variance).
__global__ void __launch_bounds__(256) k_svgf_variance(const float4* __restrict__ integrated,
                                                       const float4* __restrict__ moments,
                                                       const float4* __restrict__ dnCur, float4* __restrict__ out,
                                                       SvgfParams p) {
    int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
    if (x >= (int)p.width || y >= (int)p.height) return;
    size_t i = (size_t)y * p.width + x;
    float4 c = integrated[i], m = moments[i];
    float var;
    if (m.z >= 4.0f) {
        var = fmaxf(0.0f, m.y - m.x * m.x);
    } else {
        constexpr float kLog2e = 1.4426950408889634f;
        float4 dp = dnCur[i];
        float s1 = 0.0f, s2 = 0.0f, sw = 0.0f;
        // Gaussian x depth x normal weights as one exp2 (as in the a-trous pass)
        const float g2 = kLog2e / (2.0f * p.varianceSigma * p.varianceSigma), dz2 = kLog2e / p.depthWeight;
        for (int dy = -p.varianceRadius; dy <= p.varianceRadius; ++dy)
            for (int dx = -p.varianceRadius; dx <= p.varianceRadius; ++dx) {
                int qx = x + dx, qy = y + dy;
                if (!inside(qx, qy, p)) continue;
                size_t j = (size_t)qy * p.width + qx;
                float4 mq = moments[j];
                float4 dq = dnCur[j];
                float cosn = fmaxf(0.0f, dp.y * dq.y + dp.z * dq.z + dp.w * dq.w);
                float w = exp2f(-(float)(dx * dx + dy * dy) * g2 - fabsf(dp.x - dq.x) * dz2 +
                                p.normalWeight * __log2f(cosn));
                s1 += w * mq.x;
                s2 += w * mq.y;
                sw += w;
            }
        float inv = sw > 0.0f ? 1.0f / sw : 0.0f;
        float m1 = s1 * inv, m2 = s2 * inv;
        var = fmaxf(0.0f, m2 - m1 * m1) * (4.0f / fmaxf(m.z, 1.0f));
    }
    out[i] = make_float4(c.x, c.y, c.z, var);
}

// One a-trous pass over (rgb, variance) with step `p.step`.  The tap weight
// Gaussian(k) * depth * normal * luminance terms is evaluated as one
// exp2 of the summed exponents (the normal term's power through one log2):
// two special-function operations per tap.
__global__ void __launch_bounds__(256) k_svgf_atrous(const float4* __restrict__ src, const float4* __restrict__ dnCur,
                                                     float4* __restrict__ dst, float4* __restrict__ history,
                                                     SvgfParams p) {
    constexpr float kLog2e = 1.4426950408889634f;
    int x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
    if (x >= (int)p.width || y >= (int)p.height) return;
    size_t i = (size_t)y * p.width + x;
    float4 cp = src[i];
    float4 dp = dnCur[i];
    // 3x3 Gaussian prefilter of the variance (three distinct weights)
    float gpre = 1.0f / (2.0f * p.prefilterSigma * p.prefilterSigma);
    const float wpre[3] = {1.0f, __expf(-gpre), __expf(-2.0f * gpre)};
    float vs = 0.0f, vw = 0.0f;
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
            int qx = x + dx, qy = y + dy;
            if (!inside(qx, qy, p)) continue;
            float w = wpre[dx * dx + dy * dy];
            vs += w * src[(size_t)qy * p.width + qx].w;
            vw += w;
        }
    float sigmaL = sqrtf(fmaxf(vs / vw, 0.0f));
    float lumScale = 1.0f / (p.luminanceWeight * sigmaL + 1.0e-6f);
    float lp = luminance(make_float3(cp.x, cp.y, cp.z));
    // exponents in log2 units
    const float gb2 = kLog2e / (2.0f * p.bilateralSigma * p.bilateralSigma);
    const float dz2 = kLog2e / p.depthWeight, dl2 = kLog2e * lumScale;
    float3 sc = make_float3(0.0f, 0.0f, 0.0f);
    float sv = 0.0f, sw = 0.0f;
    for (int ky = -p.radius; ky <= p.radius; ++ky)
        for (int kx = -p.radius; kx <= p.radius; ++kx) {
            int qx = x + kx * p.step, qy = y + ky * p.step;
            if (!inside(qx, qy, p)) continue;
            size_t j = (size_t)qy * p.width + qx;
            float4 cq = src[j];
            float4 dq = dnCur[j];
            float lq = luminance(make_float3(cq.x, cq.y, cq.z));
            float cosn = fmaxf(0.0f, dp.y * dq.y + dp.z * dq.z + dp.w * dq.w);
            float e = -(float)(kx * kx + ky * ky) * gb2 - fabsf(dp.x - dq.x) * dz2 - fabsf(lp - lq) * dl2 +
                      p.normalWeight * __log2f(cosn);
            float w = exp2f(e);
            sc.x += w * cq.x;
            sc.y += w * cq.y;
            sc.z += w * cq.z;
            sv += w * w * cq.w;
            sw += w;
        }
    float inv = sw > 0.0f ? 1.0f / sw : 0.0f;
    float4 o = sw > 0.0f ? make_float4(sc.x * inv, sc.y * inv, sc.z * inv, sv * inv * inv) : cp;
    dst[i] = o;
    if (p.writeHistory) history[i] = make_float4(o.x, o.y, o.z, 0.0f);
}

// copySVGFOutputKernel: non-finite results fall back to the input, negative
// channels clamp to 0, alpha from the input.
__global__ void __launch_bounds__(256) k_svgf_copy(const float4* __restrict__ denoised,
                                                   const float4* __restrict__ original, float4* __restrict__ out,
                                                   uint32_t width, uint32_t height) {
    uint32_t x = blockIdx.x * 16 + threadIdx.x % 16, y = blockIdx.y * 16 + threadIdx.x / 16;
    if (x >= width || y >= height) return;
    size_t i = (size_t)y * width + x;
    float4 f = denoised[i], o = original[i];
    if (!(isfinite(f.x) && isfinite(f.y) && isfinite(f.z))) f = o;
    out[i] = make_float4(fmaxf(f.x, 0.0f), fmaxf(f.y, 0.0f), fmaxf(f.z, 0.0f), o.w);
}

dim3 tiles(uint32_t w, uint32_t h) { return dim3((w + 15) / 16, (h + 15) / 16); }

// The planes are read and written as float4.
bool aligned16(const void* p) { return reinterpret_cast<uintptr_t>(p) % 16u == 0u; }

}  // namespace

struct Svgf {
    uint32_t width = 0, height = 0;
    float4* block = nullptr;  // all planes below, one allocation
    float4* dn[2] = {nullptr, nullptr};
    float4* color[2] = {nullptr, nullptr};    // history colour (first a-trous pass)
    float4* moments[2] = {nullptr, nullptr};  // mu1, mu2, history length
    float4* integrated = nullptr;
    float4* work[2] = {nullptr, nullptr};
    int cur = 0;
    bool hasHistory = false;
};

}  // namespace dk

using dk::fail;

extern "C" {

int dk_svgf_create(uint32_t width, uint32_t height, dk_svgf** out) {
    if (!out || width == 0 || height == 0) return fail(DK_ERROR_INVALID_ARGUMENT, "dk_svgf_create");
    *out = nullptr;
    int rc = dk::ensureDevice();
    if (rc != DK_OK) return rc;
    auto* s = new dk::Svgf();
    s->width = width;
    s->height = height;
    size_t n = (size_t)width * height;
    if (cudaMalloc(&s->block, 9 * n * sizeof(float4)) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return fail(DK_ERROR_OUT_OF_MEMORY, "dk_svgf_create: device allocation");
    }
    float4* p = s->block;
    for (int k = 0; k < 2; ++k) s->dn[k] = p + (size_t)k * n;
    for (int k = 0; k < 2; ++k) s->color[k] = p + (size_t)(2 + k) * n;
    for (int k = 0; k < 2; ++k) s->moments[k] = p + (size_t)(4 + k) * n;
    s->integrated = p + 6 * n;
    for (int k = 0; k < 2; ++k) s->work[k] = p + (size_t)(7 + k) * n;
    *out = reinterpret_cast<dk_svgf*>(s);
    return DK_OK;
}

int dk_svgf_reset(dk_svgf* svgf) {
    auto* s = reinterpret_cast<dk::Svgf*>(svgf);
    if (!s) return fail(DK_ERROR_INVALID_ARGUMENT, "dk_svgf_reset: null");
    s->hasHistory = false;
    return DK_OK;
}

int dk_svgf_denoise(dk_svgf* svgf, const float* beauty, const float* depth, const float* normal, const float* motion,
                    float* out, const dk_spatial_denoise_settings* settings, void* stream) {
    auto* s = reinterpret_cast<dk::Svgf*>(svgf);
    if (!s || !beauty || !depth || !normal || !motion || !out || !settings)
        return fail(DK_ERROR_INVALID_ARGUMENT, "dk_svgf_denoise: null argument");
    if (!dk::aligned16(beauty) || !dk::aligned16(depth) || !dk::aligned16(normal) || !dk::aligned16(motion) ||
        !dk::aligned16(out))
        return fail(DK_ERROR_INVALID_ARGUMENT, "dk_svgf_denoise: planes must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint32_t W = s->width, H = s->height;
    dim3 g = dk::tiles(W, H);
    auto f4 = [](const float* q) { return reinterpret_cast<const float4*>(q); };
    // AppleSVGFDenoiser.configure(settings:) (Denoiser.swift:227-237)
    dk::SvgfParams p{};
    p.width = W;
    p.height = H;
    int r = (int)std::max(1u, std::min(settings->radius, 4u));
    p.radius = r;
    p.varianceRadius = r;
    p.depthWeight = std::max(settings->depth_sigma, 0.0001f);
    p.normalWeight = std::max(1.0f, std::min(512.0f, 1.0f / std::max(settings->normal_sigma, 0.0001f) * 24.0f));
    p.luminanceWeight = std::max(settings->color_sigma, 0.0001f);
    p.bilateralSigma = 1.2f;
    p.varianceSigma = 2.0f;
    p.prefilterSigma = 1.33f;
    p.alpha = 0.2f;
    p.alphaMoments = 0.2f;
    p.hasHistory = s->hasHistory ? 1 : 0;
    const int iterations = (int)std::max(1u, std::min(settings->iterations, 5u));
    const int c = s->cur, prev = 1 - c;
    dk::k_svgf_pack<<<g, 256, 0, st>>>(f4(depth), f4(normal), s->dn[c], W, H);
    dk::k_svgf_temporal<<<g, 256, 0, st>>>(f4(beauty), f4(motion), s->dn[c], s->dn[prev], s->color[prev],
                                           s->moments[prev], s->integrated, s->moments[c], p);
    dk::k_svgf_variance<<<g, 256, 0, st>>>(s->integrated, s->moments[c], s->dn[c], s->work[0], p);
    int src = 0;
    for (int it = 0; it < iterations; ++it) {
        p.step = 1 << it;
        p.writeHistory = it == 0;
        dk::k_svgf_atrous<<<g, 256, 0, st>>>(s->work[src], s->dn[c], s->work[1 - src], s->color[c], p);
        src = 1 - src;
    }
    dk::k_svgf_copy<<<g, 256, 0, st>>>(s->work[src], f4(beauty), reinterpret_cast<float4*>(out), W, H);
    DK_CUDA(cudaGetLastError(), "svgf launch");
    s->cur = prev;
    s->hasHistory = true;
    return DK_OK;
}

int dk_svgf_read_state(dk_svgf* svgf, int which, float* deviceRgba, size_t pixelCount, void* stream) {
    auto* s = reinterpret_cast<dk::Svgf*>(svgf);
    if (!s || !deviceRgba) return fail(DK_ERROR_INVALID_ARGUMENT, "dk_svgf_read_state: null argument");
    if (pixelCount != (size_t)s->width * s->height)
        return fail(DK_ERROR_INVALID_ARGUMENT, "pixel_count must equal width*height");
    if (which < 0 || which > 2) return fail(DK_ERROR_INVALID_ARGUMENT, "dk_svgf_read_state: which is 0, 1 or 2");
    const int last = 1 - s->cur;  // the frame denoised last
    const float4* src = which == 0 ? s->color[last] : which == 1 ? s->moments[last] : s->dn[last];
    DK_CUDA(cudaMemcpyAsync(deviceRgba, src, pixelCount * sizeof(float4), cudaMemcpyDeviceToDevice,
                            static_cast<cudaStream_t>(stream)),
            "svgf state copy");
    return DK_OK;
}

int dk_svgf_destroy(dk_svgf* svgf) {
    auto* s = reinterpret_cast<dk::Svgf*>(svgf);
    if (!s) return DK_OK;
    cudaDeviceSynchronize();
    cudaFree(s->block);
    delete s;
    return DK_OK;
}

int dk_svgf_pack_depth_normal(const float* depth, const float* normal, float* depthNormal, uint32_t width,
                              uint32_t height, void* stream) {
    if (!depth || !normal || !depthNormal || !dk::aligned16(depth) || !dk::aligned16(normal) ||
        !dk::aligned16(depthNormal))
        return fail(DK_ERROR_INVALID_ARGUMENT, "dk_svgf_pack_depth_normal: null or misaligned plane");
    if (width == 0 || height == 0) return DK_OK;
    dk::k_svgf_pack<<<dk::tiles(width, height), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const float4*>(depth), reinterpret_cast<const float4*>(normal),
        reinterpret_cast<float4*>(depthNormal), width, height);
    DK_CUDA(cudaGetLastError(), "svgf pack launch");
    return DK_OK;
}

int dk_svgf_copy_output(const float* denoised, const float* original, float* out, uint32_t width, uint32_t height,
                        void* stream) {
    if (!denoised || !original || !out || !dk::aligned16(denoised) || !dk::aligned16(original) || !dk::aligned16(out))
        return fail(DK_ERROR_INVALID_ARGUMENT, "dk_svgf_copy_output: null or misaligned plane");
    if (width == 0 || height == 0) return DK_OK;
    dk::k_svgf_copy<<<dk::tiles(width, height), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const float4*>(denoised), reinterpret_cast<const float4*>(original),
        reinterpret_cast<float4*>(out), width, height);
    DK_CUDA(cudaGetLastError(), "svgf copy launch");
    return DK_OK;
}

}  // extern "C"
