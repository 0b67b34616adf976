// Display encoding of render outputs and PNG export.
//
// PNGWriter.visualizedRGBA8Pixels (Sources/DenrimRendererKit/Image/PNGWriter.swift:35-53)
// on the device: every output kind becomes 8-bit RGBA the way the reference's
// PNG export shows it --
//   beauty:         exposure 0.8, the ACES fit, gamma 1/2.2, alpha kept (:146-152, :158-160)
//   depth:          finite positive depths mapped to 0.1..1 of their range, grey (:83-116)
//   normal, albedo: clamp + gamma 1/2.2, albedo keeps alpha (:153-156)
//   material/object ID: rounded ID through the reference's integer hash to a colour (:118-138, :162-174)
//   motion vector:  x, y over max(max |x|, |y|, 1) to 0..255 around 128 (:140-158, :176-178)
// Each formula is evaluated in the reference's operation order with
// explicitly rounded float operations (no contraction into FMAs), so the
// only difference from the reference's bytes can come from `pow` in the
// gamma curve (a last-bit difference in powf can move a byte by one).
// Depth and motion vectors need one statistic of the whole image (depth
// range, largest motion component): a reduction kernel writes it to a
// 16-byte workspace before the encoding kernel runs.
//
// The PNG writer (PNGWriter.write, :55-70) emits an 8-bit RGBA image with
// filter 0 rows in stored (uncompressed) deflate blocks.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/denrim_cuda.h"
#include "dk_math.cuh"

namespace dk {
void setLastError(const std::string& message);  // dk_host.cu: the dk_last_error_message() slot
}

namespace dk {
namespace {

// Workspace (DK_ENCODE_WORKSPACE_BYTES): min and max finite positive depth
// (float bits; positive floats order as their bits), largest motion
// component (float bits), count of finite positive depths.
static_assert(DK_ENCODE_WORKSPACE_BYTES >= 4 * sizeof(uint32_t), "encode workspace");

__global__ void k_image_init(uint32_t* ws) {
    ws[0] = 0x7f800000u;  // +inf
    ws[1] = 0u;
    ws[2] = 0u;
    ws[3] = 0u;
}

__global__ void __launch_bounds__(256) k_image_stats(const float4* px, uint32_t n, int kind, uint32_t* ws) {
    uint32_t lo = 0x7f800000u, hi = 0u, mag = 0u, cnt = 0u;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 p = px[i];
        if (kind == DK_OUTPUT_DEPTH) {
            if (isfinite(p.x) && p.x > 0.0f) {  // encodeDepthPixels filter (:84-86)
                uint32_t b = __float_as_uint(p.x);
                lo = min(lo, b);
                hi = max(hi, b);
                ++cnt;
            }
        } else {  // motion vectors: max(partial, max(|r|, |g|)) from 0 (:141-143)
            float m = fmaxf(fabsf(p.x), fabsf(p.y));
            if (m > 0.0f) mag = max(mag, __float_as_uint(m));
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        mag = max(mag, __shfl_xor_sync(0xffffffffu, mag, o));
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (cnt) {
            atomicMin(&ws[0], lo);
            atomicMax(&ws[1], hi);
            atomicAdd(&ws[3], cnt);
        }
        if (mag) atomicMax(&ws[2], mag);
    }
}

// UInt8(max(0, min(255, v))) of the reference: clamp, then truncate.
__device__ __forceinline__ uint32_t toByte(float v) {
    return (uint32_t)fmaxf(0.0f, fminf(255.0f, v));
}

__device__ __forceinline__ float gammaCurve(float v) {  // pow(max(0, min(1, v)), 1 / 2.2)
    return powf(fmaxf(0.0f, fminf(1.0f, v)), 1.0f / 2.2f);
}

// tonemap (:146-152)
__device__ __forceinline__ uint32_t tonemapByte(float linear) {
    float e = ex::mul(fmaxf(0.0f, linear), 0.8f);
    float num = ex::mul(e, ex::add(ex::mul(2.51f, e), 0.03f));
    float den = ex::add(ex::mul(e, ex::add(ex::mul(2.43f, e), 0.59f)), 0.14f);
    return toByte(ex::mul(gammaCurve(ex::div(num, den)), 255.0f));
}

// encodeDisplayLinear (:153-156), encodeAlpha (:158-160), encodeSigned (:176-178)
__device__ __forceinline__ uint32_t linearByte(float v) { return toByte(ex::mul(gammaCurve(v), 255.0f)); }
__device__ __forceinline__ uint32_t alphaByte(float a) { return toByte(ex::mul(a, 255.0f)); }
__device__ __forceinline__ uint32_t signedByte(float v) {
    return toByte(ex::mul(ex::add(ex::mul(v, 0.5f), 0.5f), 255.0f));
}

// colorForID (:162-174): a 32-bit integer hash to three bytes in 64..191.
__device__ __forceinline__ uint32_t idColor(uint32_t id) {
    uint32_t h = id * 747796405u + 2891336453u;
    h = ((h >> ((h >> 28) + 4u)) ^ h) * 277803737u;
    h = (h >> 22) ^ h;
    return (64u + (h & 0x7fu)) | ((64u + ((h >> 8) & 0x7fu)) << 8) | ((64u + ((h >> 16) & 0x7fu)) << 16) |
           0xff000000u;
}

__device__ __forceinline__ uint32_t pack(uint32_t r, uint32_t g, uint32_t b, uint32_t a) {
    return r | (g << 8) | (b << 16) | (a << 24);
}

__global__ void __launch_bounds__(256) k_encode_rgba8(const float4* px, uint32_t n, int kind, const uint32_t* ws,
                                                      uint32_t* out) {
    const float dLo = __uint_as_float(ws[0]), dHi = __uint_as_float(ws[1]);
    const bool anyDepth = ws[3] != 0u;
    const float dRange = ex::sub(dHi, dLo);
    const float scale = fmaxf(__uint_as_float(ws[2]), 1.0f);  // max(maxMagnitude, 1)
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = px[i];
        uint32_t v;
        switch (kind) {
            case DK_OUTPUT_BEAUTY:
                v = pack(tonemapByte(p.x), tonemapByte(p.y), tonemapByte(p.z), alphaByte(p.w));
                break;
            case DK_OUTPUT_DEPTH: {
                if (!anyDepth) {
                    v = 0u;  // no finite positive depth: all bytes zero (:88-90)
                } else if (!(isfinite(p.x) && p.x > 0.0f)) {
                    v = pack(0u, 0u, 0u, 255u);
                } else {
                    float t = dRange <= 1.1920929e-7f ? 1.0f : ex::div(ex::sub(p.x, dLo), dRange);
                    uint32_t g = toByte(ex::mul(ex::add(0.1f, ex::mul(t, 0.9f)), 255.0f));
                    v = pack(g, g, g, 255u);
                }
                break;
            }
            case DK_OUTPUT_NORMAL:
                v = pack(linearByte(p.x), linearByte(p.y), linearByte(p.z), 255u);
                break;
            case DK_OUTPUT_ALBEDO:
                v = pack(linearByte(p.x), linearByte(p.y), linearByte(p.z), alphaByte(p.w));
                break;
            case DK_OUTPUT_MATERIAL_ID:
            case DK_OUTPUT_OBJECT_ID: {
                float r = roundf(p.x);  // Int(pixel.r.rounded()): nearest, ties away from zero
                v = (r > 0.0f) ? idColor((uint32_t)fminf(r, 4294967040.0f)) : pack(0u, 0u, 0u, 255u);
                break;
            }
            default:  // DK_OUTPUT_MOTION_VECTOR
                v = pack(signedByte(ex::div(p.x, scale)), signedByte(ex::div(p.y, scale)), 128u, 255u);
                break;
        }
        out[i] = v;
    }
}

int fail(int code, const std::string& msg) {
    setLastError(msg);
    return code;
}

// ---------------------------------------------------------------- PNG ----
uint32_t crc32(const uint8_t* p, size_t n, uint32_t c = 0xffffffffu) {
    static const std::vector<uint32_t> table = [] {
        std::vector<uint32_t> t(256);
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t v = i;
            for (int k = 0; k < 8; ++k) v = (v & 1u) ? 0xedb88320u ^ (v >> 1) : v >> 1;
            t[i] = v;
        }
        return t;
    }();
    for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xffu] ^ (c >> 8);
    return c;
}

void put32(std::vector<uint8_t>& b, uint32_t v) {
    b.push_back((uint8_t)(v >> 24));
    b.push_back((uint8_t)(v >> 16));
    b.push_back((uint8_t)(v >> 8));
    b.push_back((uint8_t)v);
}

void chunk(std::vector<uint8_t>& file, const char* type, const std::vector<uint8_t>& data) {
    put32(file, (uint32_t)data.size());
    size_t start = file.size();
    file.insert(file.end(), type, type + 4);
    file.insert(file.end(), data.begin(), data.end());
    put32(file, crc32(&file[start], file.size() - start) ^ 0xffffffffu);
}

}  // namespace

int writePng(const char* path, const uint8_t* rgba, uint32_t w, uint32_t h) {
    // Scanlines: filter byte 0, then the row's RGBA bytes.
    const size_t row = (size_t)w * 4;
    std::vector<uint8_t> raw;
    raw.reserve((row + 1) * h);
    for (uint32_t y = 0; y < h; ++y) {
        raw.push_back(0);
        raw.insert(raw.end(), rgba + y * row, rgba + (y + 1) * row);
    }
    // zlib stream of stored deflate blocks (RFC 1950 / 1951) with its Adler-32.
    std::vector<uint8_t> z = {0x78, 0x01};
    size_t off = 0;
    do {
        size_t len = std::min<size_t>(65535, raw.size() - off);
        bool last = off + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)len);
        z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)~len);
        z.push_back((uint8_t)(~len >> 8));
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + len);
        off += len;
    } while (off < raw.size());
    uint32_t a = 1, b = 0;
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    put32(z, (b << 16) | a);
    std::vector<uint8_t> file = {0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
    std::vector<uint8_t> ihdr;
    put32(ihdr, w);
    put32(ihdr, h);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8-bit RGBA, deflate, filter 0, no interlace
    chunk(file, "IHDR", ihdr);
    chunk(file, "IDAT", z);
    chunk(file, "IEND", {});
    FILE* f = fopen(path, "wb");
    if (!f) return fail(DK_ERROR_EXPORT_FAILED, std::string("Could not write PNG to ") + path + ".");
    size_t wrote = fwrite(file.data(), 1, file.size(), f);
    int closed = fclose(f);
    if (wrote != file.size() || closed != 0)
        return fail(DK_ERROR_EXPORT_FAILED, std::string("Could not write PNG to ") + path + ".");
    return DK_OK;
}

cudaError_t encodeRgba8(const float4* px, uint32_t n, int kind, uint32_t* ws, uint32_t* out, cudaStream_t st) {
    int grid = (int)std::min<uint32_t>((n + 255u) / 256u, 152u * 16u);
    if (grid < 1) grid = 1;
    if (kind == DK_OUTPUT_DEPTH || kind == DK_OUTPUT_MOTION_VECTOR) {
        k_image_init<<<1, 1, 0, st>>>(ws);
        k_image_stats<<<grid, 256, 0, st>>>(px, n, kind, ws);
    }
    k_encode_rgba8<<<grid, 256, 0, st>>>(px, n, kind, ws, out);
    return cudaGetLastError();
}

}  // namespace dk

extern "C" {

int dk_encode_rgba8(const float* pixels, uint32_t width, uint32_t height, int output, uint8_t* rgba,
                    void* workspace, void* stream) {
    if (!pixels || !rgba || !workspace) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "null argument");
    if (output < DK_OUTPUT_BEAUTY || output > DK_OUTPUT_MOTION_VECTOR)
        return dk::fail(DK_ERROR_INVALID_ARGUMENT, "unknown output kind");
    if ((reinterpret_cast<uintptr_t>(pixels) & 15u) || (reinterpret_cast<uintptr_t>(rgba) & 3u) ||
        (reinterpret_cast<uintptr_t>(workspace) & 3u))
        return dk::fail(DK_ERROR_INVALID_ARGUMENT, "pixels must be 16-byte and rgba / workspace 4-byte aligned");
    uint64_t n = (uint64_t)width * height;
    if (n == 0 || n > 0xffffffffull) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "bad image size");
    cudaError_t e = dk::encodeRgba8(reinterpret_cast<const float4*>(pixels), (uint32_t)n, output,
                                    reinterpret_cast<uint32_t*>(workspace), reinterpret_cast<uint32_t*>(rgba),
                                    reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return dk::fail(DK_ERROR_COMMAND_FAILED, std::string("encode launch: ") + cudaGetErrorString(e));
    return DK_OK;
}

int dk_write_png(const char* path, const uint8_t* rgba, uint32_t width, uint32_t height) {
    if (!path || !rgba || width == 0 || height == 0) return dk::fail(DK_ERROR_INVALID_ARGUMENT, "bad argument");
    return dk::writePng(path, rgba, width, height);
}

}  // extern "C"
