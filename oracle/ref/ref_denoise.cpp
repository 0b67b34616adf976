// Test infrastructure: host driver for the reference's simpleSpatialDenoiseKernel
// (Denoise.metal:39-115, rewritten to C++ by metal2cpp.py), dispatched over all
// texels for `iterations` passes with step width 1 << pass, as
// SimpleSpatialDenoiser.encode does (Denoising/Denoiser.swift:103-160); and for
// the SVGF helpers packSVGFDepthNormalKernel and copySVGFOutputKernel
// (Denoise.metal:117-154) dispatched over all texels once.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "denoise_ref.cpp"

extern "C" int ref_denoise_spatial(const float* beauty, const float* depth, const float* normal, const float* albedo,
                                   float* out, uint32_t width, uint32_t height, uint32_t radius, float normalSigma,
                                   float depthSigma, float albedoSigma, float colorSigma, uint32_t iterations) {
    using namespace mref;
    if (!beauty || !depth || !normal || !albedo || !out) return 1;
    const size_t n = (size_t)width * height;
    std::vector<float4> a(n), b(n);
    iterations = std::max(1u, std::min(iterations, 5u));
    auto tex = [&](const float* p) {
        return texture2d<float, access::read>{reinterpret_cast<float4*>(const_cast<float*>(p)), width, height};
    };
    texture2d<float, access::read> src = tex(beauty);
    for (uint32_t it = 0; it < iterations; ++it) {
        float4* dstPix = it == iterations - 1 ? reinterpret_cast<float4*>(out) : (it % 2 == 0 ? a.data() : b.data());
        texture2d<float, access::write> dst{dstPix, width, height};
        GPUDenoiseConstants c{};
        c.width = width;
        c.height = height;
        c.radius = std::max(1u, std::min(radius, 2u));
        c.normalSigma = std::max(normalSigma, 0.0001f);
        c.depthSigma = std::max(depthSigma, 0.0001f);
        c.albedoSigma = std::max(albedoSigma, 0.0001f);
        c.colorSigma = std::max(colorSigma, 0.0001f);
        c.stepWidth = 1u << it;
        for (uint32_t y = 0; y < height; ++y)
            for (uint32_t x = 0; x < width; ++x)
                simpleSpatialDenoiseKernel(src, tex(depth), tex(normal), tex(albedo), dst, c, uint2(x, y));
        src = texture2d<float, access::read>{dstPix, width, height};
    }
    return 0;
}

extern "C" int ref_svgf_pack_depth_normal(const float* depth, const float* normal, float* out, uint32_t width,
                                          uint32_t height) {
    using namespace mref;
    if (!depth || !normal || !out) return 1;
    auto rd = [&](const float* p) {
        return texture2d<float, access::read>{reinterpret_cast<float4*>(const_cast<float*>(p)), width, height};
    };
    texture2d<float, access::write> dst{reinterpret_cast<float4*>(out), width, height};
    for (uint32_t y = 0; y < height; ++y)
        for (uint32_t x = 0; x < width; ++x) packSVGFDepthNormalKernel(rd(depth), rd(normal), dst, uint2(x, y));
    return 0;
}

extern "C" int ref_svgf_copy_output(const float* denoised, const float* original, float* out, uint32_t width,
                                    uint32_t height) {
    using namespace mref;
    if (!denoised || !original || !out) return 1;
    auto rd = [&](const float* p) {
        return texture2d<float, access::read>{reinterpret_cast<float4*>(const_cast<float*>(p)), width, height};
    };
    texture2d<float, access::write> dst{reinterpret_cast<float4*>(out), width, height};
    for (uint32_t y = 0; y < height; ++y)
        for (uint32_t x = 0; x < width; ++x) copySVGFOutputKernel(rd(denoised), rd(original), dst, uint2(x, y));
    return 0;
}
