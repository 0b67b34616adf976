// Test infrastructure: the CPU oracle for the path-tracing hot path.
// Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may use
// anything under oracle/; the product never links or calls it.
//
// Vector helpers with the arithmetic of the Metal Shading Language built-ins as
// the reference shader uses them (Sources/DenrimRendererKit/Resources/Shaders/
// PathTrace.metal).  Every helper spells out its operation order, so the FP32
// build, compiled with -ffp-contract=off, is the IEEE definition the CUDA
// kernels reproduce for the bit-exact outputs (RNG, hit selection, depth,
// normal, IDs).  `real` is float in the FP32 build and double in the FP64 one.
#pragma once
#include <cmath>
#include <cstdint>

#include "../include/denrim_cuda.h"

#ifndef ORACLE_REAL
#define ORACLE_REAL float
#endif
typedef ORACLE_REAL real;

#define K(x) ((real)(x))

namespace om {

struct V2 { real x, y; };
struct V3 { real x, y, z; };
struct V4 { real x, y, z, w; V3 xyz() const { return {x, y, z}; } V2 xy() const { return {x, y}; } };

static inline V2 v2(real x, real y) { return {x, y}; }
static inline V3 v3(real x, real y, real z) { return {x, y, z}; }
static inline V3 v3(real s) { return {s, s, s}; }
static inline V4 v4(real x, real y, real z, real w) { return {x, y, z, w}; }
static inline V4 v4(V3 a, real w) { return {a.x, a.y, a.z, w}; }

static inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
static inline V3 operator*(V3 a, real s) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 operator*(real s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
static inline V3 operator/(V3 a, real s) { return {a.x / s, a.y / s, a.z / s}; }
static inline V3 operator/(real s, V3 a) { return {s / a.x, s / a.y, s / a.z}; }
static inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
static inline V3& operator+=(V3& a, V3 b) { a = a + b; return a; }
static inline V3& operator*=(V3& a, V3 b) { a = a * b; return a; }
static inline V3& operator*=(V3& a, real s) { a = a * s; return a; }
static inline V3& operator/=(V3& a, real s) { a = a / s; return a; }
static inline V2 operator+(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
static inline V2 operator-(V2 a, V2 b) { return {a.x - b.x, a.y - b.y}; }
static inline V2 operator*(V2 a, real s) { return {a.x * s, a.y * s}; }
static inline V2 operator*(real s, V2 a) { return {s * a.x, s * a.y}; }
static inline V4 operator+(V4 a, V4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
static inline V4 operator-(V4 a, V4 b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
static inline V4 operator*(V4 a, V4 b) { return {a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }
static inline V4 operator*(V4 a, real s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }

// Metal min/max are fmin/fmax (a NaN operand yields the other operand).
static inline real mn(real a, real b) { return std::fmin(a, b); }
static inline real mx(real a, real b) { return std::fmax(a, b); }
static inline V3 mn(V3 a, V3 b) { return {mn(a.x, b.x), mn(a.y, b.y), mn(a.z, b.z)}; }
static inline V3 mx(V3 a, V3 b) { return {mx(a.x, b.x), mx(a.y, b.y), mx(a.z, b.z)}; }
static inline real clampf(real x, real lo, real hi) { return mn(mx(x, lo), hi); }
static inline V3 clamp3(V3 x, V3 lo, V3 hi) { return mn(mx(x, lo), hi); }
static inline real dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline real length(V3 a) { return std::sqrt(dot(a, a)); }
// normalize(v) = v * (1 / sqrt(dot(v, v))) with correctly rounded sqrt and divide.
static inline V3 normalize(V3 a) { real s = K(1.0) / std::sqrt(dot(a, a)); return a * s; }
static inline real mixf(real a, real b, real t) { return a + (b - a) * t; }
static inline V3 mix3(V3 a, V3 b, real t) { return a + (b - a) * t; }
static inline V4 mix4(V4 a, V4 b, real t) { return a + (b - a) * t; }
static inline V3 reflect(V3 i, V3 n) { return i - (K(2.0) * dot(n, i)) * n; }
static inline V3 refract(V3 i, V3 n, real eta) {
    real d = dot(n, i);
    real k = K(1.0) - eta * eta * (K(1.0) - d * d);
    if (k < K(0.0)) return v3(K(0.0));
    return eta * i - (eta * d + std::sqrt(k)) * n;
}
static inline real fractf(real x) {
    return mn(x - std::floor(x), (real)0x1.fffffep-1f);
}
static inline real smoothstepf(real e0, real e1, real x) {
    real t = clampf((x - e0) / (e1 - e0), K(0.0), K(1.0));
    return t * t * (K(3.0) - K(2.0) * t);
}
static inline real maxComponent(V3 v) { return mx(v.x, mx(v.y, v.z)); }
static inline bool allFinite(V3 v) { return std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z); }
static inline V3 exp3(V3 v) { return {std::exp(v.x), std::exp(v.y), std::exp(v.z)}; }
static inline V3 log3(V3 v) { return {std::log(v.x), std::log(v.y), std::log(v.z)}; }
static inline V3 abs3(V3 v) { return {std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)}; }

static inline V3 ld3(const dk_float4& f) { return {(real)f.x, (real)f.y, (real)f.z}; }
static inline V4 ld4(const dk_float4& f) { return {(real)f.x, (real)f.y, (real)f.z, (real)f.w}; }

}  // namespace om
