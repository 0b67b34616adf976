// Test infrastructure: a C++20 stand-in for the subset of the Metal Shading
// Language that the reference path tracer's compute kernel uses, so that the
// reference shader source itself (after the mechanical rewrite done by
// metal2cpp.py) compiles with g++ and runs on the host as a per-pixel loop.
// Only tests/, __graft_entry__ and bench.py's reference/cpu-baseline legs use
// what is built from it; the product never links it.
//
// Arithmetic conventions are the ones the CPU restatement in oracle/ uses
// (oracle_math.hpp), so a comparison of the two checks the restatement of the
// shader's logic, not Apple's built-in implementations (which cannot run here):
//   min/max on floats = fmin/fmax, clamp = min(max(x, lo), hi),
//   mix(a, b, t) = a + (b - a) * t, normalize(v) = v * (1 / sqrt(dot(v, v))),
//   fract(x) = min(x - floor(x), 0x1.fffffep-1), smoothstep as in the MSL spec,
//   float4x4 * float4 = ((c0 * v.x + c1 * v.y) + c2 * v.z) + c3 * v.w.
#pragma once
#include <atomic>
#include <cmath>
#include <cstdint>
#include <type_traits>

#define kernel
#define device
#define constant const
#define thread
#define threadgroup

namespace mref {

typedef unsigned int uint;
template <class T> using S = std::type_identity_t<T>;

template <class T> struct vec2;
template <class T> struct vec3;
template <class T> struct vec4;

template <class T> struct vec2 {
    T x, y;
    vec2() = default;
    constexpr vec2(T a, T b) : x(a), y(b) {}
    explicit constexpr vec2(T s) : x(s), y(s) {}
    template <class U> explicit constexpr vec2(vec2<U> o) : x(T(o.x)), y(T(o.y)) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
};

template <class T> struct vec3 {
    T x, y, z;
    vec3() = default;
    constexpr vec3(T a, T b, T c) : x(a), y(b), z(c) {}
    explicit constexpr vec3(T s) : x(s), y(s), z(s) {}
    constexpr vec3(vec2<T> a, T c) : x(a.x), y(a.y), z(c) {}
    constexpr vec3(T a, vec2<T> b) : x(a), y(b.x), z(b.y) {}
    template <class U> explicit constexpr vec3(vec3<U> o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
    vec2<T> xy() const { return {x, y}; }
    vec2<T> xz() const { return {x, z}; }
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
};

template <class T> struct alignas(sizeof(T) * 4) vec4 {
    T x, y, z, w;
    vec4() = default;
    constexpr vec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    explicit constexpr vec4(T s) : x(s), y(s), z(s), w(s) {}
    constexpr vec4(vec3<T> a, T d) : x(a.x), y(a.y), z(a.z), w(d) {}
    constexpr vec4(T a, vec3<T> b) : x(a), y(b.x), z(b.y), w(b.z) {}
    constexpr vec4(vec2<T> a, vec2<T> b) : x(a.x), y(a.y), z(b.x), w(b.y) {}
    constexpr vec4(vec2<T> a, T c, T d) : x(a.x), y(a.y), z(c), w(d) {}
    template <class U> explicit constexpr vec4(vec4<U> o) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(o.w)) {}
    vec3<T> xyz() const { return {x, y, z}; }
    vec2<T> xy() const { return {x, y}; }
    void set_xyz(vec3<T> v) { x = v.x; y = v.y; z = v.z; }
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
};

typedef vec2<float> float2;
typedef vec3<float> float3;
typedef vec4<float> float4;
typedef vec2<uint> uint2;
typedef vec3<uint> uint3;
typedef vec4<uint> uint4;
typedef vec2<int> int2;
typedef vec3<int> int3;
typedef vec4<int> int4;
typedef vec2<bool> bool2;
typedef vec3<bool> bool3;
typedef vec4<bool> bool4;

// Component-wise operators (vector-vector, vector-scalar, scalar-vector).
#define MREF_BINOP(op)                                                                                    \
    template <class T> vec2<T> operator op(vec2<T> a, vec2<T> b) { return {T(a.x op b.x), T(a.y op b.y)}; } \
    template <class T> vec2<T> operator op(vec2<T> a, S<T> s) { return {T(a.x op s), T(a.y op s)}; }         \
    template <class T> vec2<T> operator op(S<T> s, vec2<T> a) { return {T(s op a.x), T(s op a.y)}; }         \
    template <class T> vec3<T> operator op(vec3<T> a, vec3<T> b) {                                         \
        return {T(a.x op b.x), T(a.y op b.y), T(a.z op b.z)};                                              \
    }                                                                                                      \
    template <class T> vec3<T> operator op(vec3<T> a, S<T> s) { return {T(a.x op s), T(a.y op s), T(a.z op s)}; } \
    template <class T> vec3<T> operator op(S<T> s, vec3<T> a) { return {T(s op a.x), T(s op a.y), T(s op a.z)}; } \
    template <class T> vec4<T> operator op(vec4<T> a, vec4<T> b) {                                         \
        return {T(a.x op b.x), T(a.y op b.y), T(a.z op b.z), T(a.w op b.w)};                               \
    }                                                                                                      \
    template <class T> vec4<T> operator op(vec4<T> a, S<T> s) {                                            \
        return {T(a.x op s), T(a.y op s), T(a.z op s), T(a.w op s)};                                       \
    }                                                                                                      \
    template <class T> vec4<T> operator op(S<T> s, vec4<T> a) {                                            \
        return {T(s op a.x), T(s op a.y), T(s op a.z), T(s op a.w)};                                       \
    }                                                                                                      \
    template <class V, class B> auto operator op##=(V& a, const B& b)->decltype(a = a op b) { return a = a op b; }
MREF_BINOP(+)
MREF_BINOP(-)
MREF_BINOP(*)
MREF_BINOP(/)
#undef MREF_BINOP

template <class T> vec2<T> operator-(vec2<T> a) { return {-a.x, -a.y}; }
template <class T> vec3<T> operator-(vec3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> vec4<T> operator-(vec4<T> a) { return {-a.x, -a.y, -a.z, -a.w}; }

#define MREF_CMP(op)                                                                                          \
    template <class T> bool2 operator op(vec2<T> a, vec2<T> b) { return {a.x op b.x, a.y op b.y}; }             \
    template <class T> bool3 operator op(vec3<T> a, vec3<T> b) { return {a.x op b.x, a.y op b.y, a.z op b.z}; } \
    template <class T> bool3 operator op(vec3<T> a, S<T> s) { return {a.x op s, a.y op s, a.z op s}; }
MREF_CMP(<)
MREF_CMP(>)
MREF_CMP(<=)
MREF_CMP(>=)
#undef MREF_CMP

inline bool all(bool2 b) { return b.x && b.y; }
inline bool all(bool3 b) { return b.x && b.y && b.z; }
inline bool any(bool3 b) { return b.x || b.y || b.z; }

// ------------------------------------------------------------- scalars ---
inline float abs(float x) { return std::fabs(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline float fabs(float x) { return std::fabs(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float rsqrt(float x) { return 1.0f / std::sqrt(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline float exp(float x) { return std::exp(x); }
inline float log(float x) { return std::log(x); }
inline float sin(float x) { return std::sin(x); }
inline float cos(float x) { return std::cos(x); }
inline float acos(float x) { return std::acos(x); }
inline float atan2(float y, float x) { return std::atan2(y, x); }
inline float floor(float x) { return std::floor(x); }
inline float round(float x) { return std::round(x); }
inline float fmod(float x, float y) { return std::fmod(x, y); }
inline float fract(float x) { return std::fmin(x - std::floor(x), 0x1.fffffep-1f); }
inline bool isfinite(float x) { return std::isfinite(x); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline uint min(uint a, uint b) { return a < b ? a : b; }
inline uint max(uint a, uint b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline uint clamp(uint x, uint lo, uint hi) { return min(max(x, lo), hi); }
inline int clamp(int x, int lo, int hi) { return min(max(x, lo), hi); }
inline float mix(float a, float b, float t) { return a + (b - a) * t; }
inline float smoothstep(float e0, float e1, float x) {
    float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// ------------------------------------------------- component-wise maps ---
#define MREF_MAP1(name)                                                                                  \
    template <class T> auto name(vec2<T> a)->vec2<decltype(name(a.x))> { return {name(a.x), name(a.y)}; } \
    template <class T> auto name(vec3<T> a)->vec3<decltype(name(a.x))> {                                  \
        return {name(a.x), name(a.y), name(a.z)};                                                         \
    }                                                                                                     \
    template <class T> auto name(vec4<T> a)->vec4<decltype(name(a.x))> {                                  \
        return {name(a.x), name(a.y), name(a.z), name(a.w)};                                              \
    }
MREF_MAP1(abs)
MREF_MAP1(fabs)
MREF_MAP1(sqrt)
MREF_MAP1(exp)
MREF_MAP1(log)
MREF_MAP1(floor)
MREF_MAP1(round)
MREF_MAP1(fract)
MREF_MAP1(isfinite)
MREF_MAP1(sin)
MREF_MAP1(cos)
MREF_MAP1(acos)
#undef MREF_MAP1

#define MREF_MAP2(name)                                                                                     \
    template <class T> vec2<T> name(vec2<T> a, vec2<T> b) { return {name(a.x, b.x), name(a.y, b.y)}; }       \
    template <class T> vec3<T> name(vec3<T> a, vec3<T> b) {                                                  \
        return {name(a.x, b.x), name(a.y, b.y), name(a.z, b.z)};                                             \
    }                                                                                                        \
    template <class T> vec4<T> name(vec4<T> a, vec4<T> b) {                                                  \
        return {name(a.x, b.x), name(a.y, b.y), name(a.z, b.z), name(a.w, b.w)};                             \
    }                                                                                                        \
    template <class T> vec3<T> name(vec3<T> a, S<T> s) { return {name(a.x, s), name(a.y, s), name(a.z, s)}; }
MREF_MAP2(min)
MREF_MAP2(max)
inline bool3 isfinite(vec3<float> v) { return {isfinite(v.x), isfinite(v.y), isfinite(v.z)}; }
MREF_MAP2(pow)
MREF_MAP2(fmod)
#undef MREF_MAP2

template <class V> V clamp(V x, V lo, V hi) { return min(max(x, lo), hi); }
template <class T> vec3<T> clamp(vec3<T> x, S<T> lo, S<T> hi) { return min(max(x, lo), hi); }
template <class T> vec2<T> mix(vec2<T> a, vec2<T> b, S<T> t) { return a + (b - a) * t; }
template <class T> vec3<T> mix(vec3<T> a, vec3<T> b, S<T> t) { return a + (b - a) * t; }
template <class T> vec4<T> mix(vec4<T> a, vec4<T> b, S<T> t) { return a + (b - a) * t; }
template <class T> vec3<T> mix(vec3<T> a, vec3<T> b, vec3<T> t) { return a + (b - a) * t; }

// ------------------------------------------------------------ geometry ---
template <class T> T dot(vec2<T> a, vec2<T> b) { return a.x * b.x + a.y * b.y; }
template <class T> T dot(vec3<T> a, vec3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> T dot(vec4<T> a, vec4<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
template <class T> vec3<T> cross(vec3<T> a, vec3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class V> auto length(V a) { return sqrt(dot(a, a)); }
template <class V> auto distance(V a, V b) { return length(a - b); }
template <class V> V normalize(V a) { return a * (1.0f / sqrt(dot(a, a))); }
inline float3 reflect(float3 i, float3 n) { return i - (2.0f * dot(n, i)) * n; }
inline float3 refract(float3 i, float3 n, float eta) {
    float d = dot(n, i);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return float3(0.0f);
    return eta * i - (eta * d + std::sqrt(k)) * n;
}

struct float4x4 {
    float4 c[4];
    float4x4() = default;
    float4x4(float4 a, float4 b, float4 d, float4 e) : c{a, b, d, e} {}
};
inline float4 operator*(const float4x4& m, float4 v) {
    return ((m.c[0] * v.x + m.c[1] * v.y) + m.c[2] * v.z) + m.c[3] * v.w;
}

// -------------------------------------------------- textures and atomics ---
enum class access { sample, read, write, read_write };

template <class T, access A = access::sample> struct texture2d {
    vec4<T>* pixels = nullptr;
    uint width = 0, height = 0;
    vec4<T> read(uint2 p) const { return pixels[(uint64_t)p.y * width + p.x]; }
    void write(vec4<T> v, uint2 p) const { pixels[(uint64_t)p.y * width + p.x] = v; }
    uint get_width() const { return width; }
    uint get_height() const { return height; }
};

struct atomic_uint {
    std::atomic<uint> value;
};
enum mref_memory_order { memory_order_relaxed };
inline uint atomic_fetch_add_explicit(atomic_uint* a, uint v, mref_memory_order) {
    return a->value.fetch_add(v, std::memory_order_relaxed);
}

}  // namespace mref
