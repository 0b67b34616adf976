// Device vector math for the sm_103a path tracer.
//
// Two families of helpers:
//   * `ex::` — every operation is an explicitly rounded IEEE op (__fadd_rn,
//     __fmul_rn, __fdiv_rn, __fsqrt_rn).  The compiler never contracts these
//     into FMAs, so camera rays, box tests, Möller-Trumbore and the hit
//     attributes reproduce the reference arithmetic bit for bit (primary
//     depth, normal, IDs and the RNG-driven control flow of the first hit).
//   * plain operators — ordinary float math (FMA contraction allowed) for the
//     BSDF and lighting code, whose results are compared statistically.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace dk {

// ------------------------------------------------------------ plain ops ---
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 f3(float s) { return make_float3(s, s, s); }
__device__ __forceinline__ float3 xyz(const float4& v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float3 operator/(float s, float3 a) { return f3(s / a.x, s / a.y, s / a.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
__device__ __forceinline__ float3& operator*=(float3& a, float3 b) { a = a * b; return a; }
__device__ __forceinline__ float3& operator*=(float3& a, float s) { a = a * s; return a; }
__device__ __forceinline__ float3& operator/=(float3& a, float s) { a = a / s; return a; }
__device__ __forceinline__ float4 operator+(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ float4 operator-(float4 a, float4 b) { return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
__device__ __forceinline__ float4 operator*(float4 a, float4 b) { return make_float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
__device__ __forceinline__ float4 operator*(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }

__device__ __forceinline__ float mn(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float mx(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ float3 mn(float3 a, float3 b) { return f3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
__device__ __forceinline__ float3 mx(float3 a, float3 b) { return f3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float3 clamp3(float3 x, float3 lo, float3 hi) { return mn(mx(x, lo), hi); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float length(float3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ float3 normalize(float3 a) { return a * (1.0f / sqrtf(dot(a, a))); }
__device__ __forceinline__ float mixf(float a, float b, float t) { return a + (b - a) * t; }
__device__ __forceinline__ float3 mix3(float3 a, float3 b, float t) { return a + (b - a) * t; }
__device__ __forceinline__ float4 mix4(float4 a, float4 b, float t) { return a + (b - a) * t; }
__device__ __forceinline__ float3 reflect(float3 i, float3 n) { return i - (2.0f * dot(n, i)) * n; }
__device__ __forceinline__ float3 refract(float3 i, float3 n, float eta) {
    float d = dot(n, i);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return f3(0.0f);
    return eta * i - (eta * d + sqrtf(k)) * n;
}
__device__ __forceinline__ float fractf(float x) { return fminf(x - floorf(x), 0x1.fffffep-1f); }
__device__ __forceinline__ float maxComponent(float3 v) { return fmaxf(v.x, fmaxf(v.y, v.z)); }
__device__ __forceinline__ bool allFinite(float3 v) { return isfinite(v.x) && isfinite(v.y) && isfinite(v.z); }
__device__ __forceinline__ float3 exp3(float3 v) { return f3(expf(v.x), expf(v.y), expf(v.z)); }
__device__ __forceinline__ float3 log3(float3 v) { return f3(logf(v.x), logf(v.y), logf(v.z)); }

// -------------------------------------------------------- exact-rounded ---
namespace ex {
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float rcp(float a) { return __frcp_rn(a); }
__device__ __forceinline__ float3 add(float3 a, float3 b) { return f3(add(a.x, b.x), add(a.y, b.y), add(a.z, b.z)); }
__device__ __forceinline__ float3 sub(float3 a, float3 b) { return f3(sub(a.x, b.x), sub(a.y, b.y), sub(a.z, b.z)); }
__device__ __forceinline__ float3 mul(float3 a, float s) { return f3(mul(a.x, s), mul(a.y, s), mul(a.z, s)); }
__device__ __forceinline__ float3 mul(float s, float3 a) { return f3(mul(s, a.x), mul(s, a.y), mul(s, a.z)); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return add(add(mul(a.x, b.x), mul(a.y, b.y)), mul(a.z, b.z)); }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return f3(sub(mul(a.y, b.z), mul(a.z, b.y)), sub(mul(a.z, b.x), mul(a.x, b.z)), sub(mul(a.x, b.y), mul(a.y, b.x)));
}
// normalize(v) = v * (1 / sqrt(dot(v, v))), both correctly rounded.
__device__ __forceinline__ float3 normalize(float3 a) {
    float s = div(1.0f, __fsqrt_rn(dot(a, a)));
    return mul(a, s);
}
}  // namespace ex

// -------------------------------------------------------------- RNG -------
// hash / randomFloat: PathTrace.metal:255-268.
__device__ __forceinline__ uint32_t hash_u32(uint32_t v) {
    v ^= v >> 16;
    v *= 0x7feb352du;
    v ^= v >> 15;
    v *= 0x846ca68bu;
    v ^= v >> 16;
    return v;
}
__device__ __forceinline__ float randomFloat(uint32_t& state) {
    state = hash_u32(state);
    return (float)(state & 0x00ffffffu) * (1.0f / 16777216.0f);  // exact: power-of-two scale
}

}  // namespace dk
