// Test infrastructure: the CPU oracle for the path-tracing hot path.
// Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may use
// anything under oracle/; the product never links or calls it.
//
// A per-pixel CPU restatement of DenrimRendererKit's `final`-quality path
// tracer, `pathTraceKernel` (Sources/DenrimRendererKit/Resources/Shaders/
// PathTrace.metal:5167-5586), and of everything it calls for triangle scenes:
// RNG, camera, binary-BVH closest hit, layered BSDF, transmission, subsurface
// and volume random walks, emissive-triangle and environment NEE with closest-
// hit shadow walks, Russian roulette, the running-mean accumulation and the
// last-sample AOVs.  Every draw of `randomFloat` happens in the left-to-right
// textual order of the reference source (the argument-evaluation order of the
// clang-based Metal compiler).  Compiled twice: ORACLE_REAL=float is the
// reference arithmetic and the timed CPU baseline; ORACLE_REAL=double is the
// FP64 error oracle.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

#include "oracle_math.hpp"
#include "oracle_params.h"

using namespace om;

namespace {

// ---------------------------------------------------------------- RNG -----
// hash / randomFloat: PathTrace.metal:255-268.
static inline uint32_t hash_u32(uint32_t value) {
    value ^= value >> 16;
    value *= 0x7feb352du;
    value ^= value >> 15;
    value *= 0x846ca68bu;
    value ^= value >> 16;
    return value;
}
static inline real randomFloat(uint32_t& state) {
    state = hash_u32(state);
    return (real)(float)(state & 0x00ffffffu) / (real)(float)0x01000000u;
}

// ---------------------------------------------------------- counters ------
// Work counters behind the algorithmic-bytes figure of the roofline.
// Query kinds: 0 extension (bounce loop), 1 shadow, 2 subsurface walk, 3 AOV.
enum {
    C_PATHS = 0, C_MATERIAL_FETCH, C_LIGHT_SAMPLES, C_ENV_SAMPLES, C_ENV_SEARCH_STEPS,
    C_MISS_ENV, C_SHADOW_QUERIES, C_BOUNCES, C_ENV_LOOKUPS,
    C_QUERIES_K0, C_QUERIES_K1, C_QUERIES_K2, C_QUERIES_K3,
    C_NODES_K0, C_NODES_K1, C_NODES_K2, C_NODES_K3,
    C_TRIS_K0, C_TRIS_K1, C_TRIS_K2, C_TRIS_K3,
    C_GRID_CELLS, C_MACRO_SKIPS, C_BRICK_TESTS, C_BRICK_MARCHES, C_MARCH_STEPS, C_BRICK_HITS, C_BRICK_SAMPLES,
    C_RANGE_CULLS,
    C_COUNT
};
struct Counters { uint64_t c[C_COUNT]; };

// ------------------------------------------------------------- types ------
struct Ray { V3 origin, direction; };

// Hit: PathTrace.metal:229-253 (the volume-field members stay zero for the
// triangle scenes this oracle renders).
struct Hit {
    bool hit;
    real t;
    V3 position;
    V3 normal;
    V2 uv;
    V3 tangent;
    V3 bitangent;
    uint32_t materialID;
    uint32_t materialID2;
    real materialBlend;
    uint32_t objectID;
    uint32_t primitiveID;
    bool frontFacing;
};

struct Material {
    V4 baseColor, emission, parameters, parameters2, specularColor, sheenColor,
        transmissionColor, parameters3, clearcoatColor, clearcoatAttenuation,
        transmissionAbsorption, thinFilm, subsurfaceColor, subsurfaceRadius,
        subsurfaceParameters, volumeScattering, volumeParameters;
};

static Material loadMaterial(const dk_material& m) {
    Material r;
    r.baseColor = ld4(m.base_color);
    r.emission = ld4(m.emission);
    r.parameters = ld4(m.parameters);
    r.parameters2 = ld4(m.parameters2);
    r.specularColor = ld4(m.specular_color);
    r.sheenColor = ld4(m.sheen_color);
    r.transmissionColor = ld4(m.transmission_color);
    r.parameters3 = ld4(m.parameters3);
    r.clearcoatColor = ld4(m.clearcoat_color);
    r.clearcoatAttenuation = ld4(m.clearcoat_attenuation);
    r.transmissionAbsorption = ld4(m.transmission_absorption);
    r.thinFilm = ld4(m.thin_film);
    r.subsurfaceColor = ld4(m.subsurface_color);
    r.subsurfaceRadius = ld4(m.subsurface_radius);
    r.subsurfaceParameters = ld4(m.subsurface_parameters);
    r.volumeScattering = ld4(m.volume_scattering);
    r.volumeParameters = ld4(m.volume_parameters);
    return r;
}

}  // namespace


namespace {

struct Ctx {
    const dk_scene* s;
    const oracle_params* p;
    Counters* cnt;
};

static inline void count(const Ctx& c, int slot, uint64_t v = 1) { c.cnt->c[slot] += v; }

// ----------------------------------------------------- sampling helpers ---
// cosineHemisphere: PathTrace.metal:270-275
static V3 cosineHemisphere(V2 u) {
    real r = std::sqrt(u.x);
    real phi = K(6.28318530718) * u.y;
    return v3(r * std::cos(phi), r * std::sin(phi), std::sqrt(mx(K(0.0), K(1.0) - u.x)));
}
// uniformDisk: PathTrace.metal:277-281
static V2 uniformDisk(V2 u) {
    real r = std::sqrt(u.x);
    real phi = K(6.28318530718) * u.y;
    return v2(r * std::cos(phi), r * std::sin(phi));
}
// uniformSphere: PathTrace.metal:283-288
static V3 uniformSphere(V2 u) {
    real z = K(1.0) - K(2.0) * u.x;
    real r = std::sqrt(mx(K(0.0), K(1.0) - z * z));
    real phi = K(6.28318530718) * u.y;
    return v3(r * std::cos(phi), r * std::sin(phi), z);
}
// orientHemisphere: PathTrace.metal:290-295
static V3 orientHemisphere(V3 local, V3 normal) {
    V3 helper = std::fabs(normal.y) < K(0.999) ? v3(0, 1, 0) : v3(1, 0, 0);
    V3 tangent = normalize(cross(helper, normal));
    V3 bitangent = cross(normal, tangent);
    return normalize(local.x * tangent + local.y * bitangent + local.z * normal);
}
// orientAroundDirection: PathTrace.metal:297-302
static V3 orientAroundDirection(V3 local, V3 direction) {
    V3 helper = std::fabs(direction.y) < K(0.999) ? v3(0, 1, 0) : v3(1, 0, 0);
    V3 tangent = normalize(cross(helper, direction));
    V3 bitangent = cross(direction, tangent);
    return normalize(local.x * tangent + local.y * bitangent + local.z * direction);
}
// sampleHenyeyGreenstein: PathTrace.metal:304-318
static V3 sampleHenyeyGreenstein(V2 u, V3 direction, real anisotropy) {
    real g = clampf(anisotropy, K(-0.95), K(0.95));
    if (std::fabs(g) < K(1e-4)) return uniformSphere(u);
    real oneMinusGSquared = K(1.0) - g * g;
    real denominator = K(1.0) - g + K(2.0) * g * u.x;
    real q = oneMinusGSquared / mx(denominator, K(1e-5));
    real cosTheta = (K(1.0) + g * g - q * q) / (K(2.0) * g);
    cosTheta = clampf(cosTheta, K(-1.0), K(1.0));
    real sinTheta = std::sqrt(mx(K(0.0), K(1.0) - cosTheta * cosTheta));
    real phi = K(6.28318530718) * u.y;
    return orientAroundDirection(v3(std::cos(phi) * sinTheta, std::sin(phi) * sinTheta, cosTheta), direction);
}
// clampSampleContribution: PathTrace.metal:324-340
static V3 clampSampleContribution(V3 c, const Ctx& ctx) {
    if (!allFinite(c)) return v3(K(0.0));
    real clampValue = mx((real)ctx.p->sample_radiance_clamp, K(0.0));
    if (clampValue <= K(0.0)) return c;
    real peak = maxComponent(c);
    if (peak <= clampValue) return c;
    return c * (clampValue / mx(peak, K(1e-5)));
}
// luminance: PathTrace.metal:342-344
static real luminance(V3 v) { return dot(v, v3(K(0.2126), K(0.7152), K(0.0722))); }

// ------------------------------------------------------ material model ----
// fresnelSchlick / thinFilmTint / fresnelSchlickThinFilm: PathTrace.metal:346-376
static V3 fresnelSchlick(real cosTheta, V3 f0) {
    real factor = std::pow(clampf(K(1.0) - cosTheta, K(0.0), K(1.0)), K(5.0));
    return f0 + (v3(K(1.0)) - f0) * factor;
}
static V3 thinFilmTint(const Material& m, real cosTheta) {
    real strength = clampf(m.thinFilm.x, K(0.0), K(1.0));
    real thickness = mx(m.thinFilm.y, K(0.0));
    if (strength <= K(0.0) || thickness <= K(0.0)) return v3(K(1.0));
    real filmIOR = mx(m.thinFilm.z, K(1.0001));
    real angle = std::pow(clampf(K(1.0) - cosTheta, K(0.0), K(1.0)), K(0.65));
    real opticalPath = K(2.0) * filmIOR * thickness * (K(0.62) + K(0.42) * angle);
    V3 wavelengths = v3(K(650.0), K(510.0), K(475.0));
    V3 phase = K(6.28318530718) * opticalPath / wavelengths;
    V3 interference = v3(K(0.62) + K(0.38) * std::cos(phase.x), K(0.62) + K(0.38) * std::cos(phase.y),
                         K(0.62) + K(0.38) * std::cos(phase.z));
    real normalizedLuminance = mx(luminance(interference), K(0.35));
    V3 tint = clamp3(interference / normalizedLuminance, v3(K(0.35)), v3(K(1.8)));
    return mix3(v3(K(1.0)), tint, strength);
}
static V3 fresnelSchlickThinFilm(real cosTheta, V3 f0, const Material& m) {
    return fresnelSchlick(cosTheta, f0) * thinFilmTint(m, cosTheta);
}
// dielectricFresnel: PathTrace.metal:378-393
static real dielectricFresnel(real cosThetaI, real etaI, real etaT) {
    cosThetaI = clampf(cosThetaI, K(0.0), K(1.0));
    real eta = etaI / etaT;
    real sinThetaTSquared = eta * eta * mx(K(0.0), K(1.0) - cosThetaI * cosThetaI);
    if (sinThetaTSquared >= K(1.0)) return K(1.0);
    real cosThetaT = std::sqrt(mx(K(0.0), K(1.0) - sinThetaTSquared));
    real parallel = ((etaT * cosThetaI) - (etaI * cosThetaT)) / mx((etaT * cosThetaI) + (etaI * cosThetaT), K(1e-5));
    real perpendicular = ((etaI * cosThetaI) - (etaT * cosThetaT)) / mx((etaI * cosThetaI) + (etaT * cosThetaT), K(1e-5));
    return clampf(K(0.5) * (parallel * parallel + perpendicular * perpendicular), K(0.0), K(1.0));
}
// dielectricF0 / materialF0 / clearcoat accessors: PathTrace.metal:395-440
static real dielectricF0(real ior_, real specularWeight) {
    real ior = mx(ior_, K(1.0));
    real f0 = (ior - K(1.0)) / (ior + K(1.0));
    return f0 * f0 * clampf(specularWeight, K(0.0), K(1.0));
}
static V3 materialF0(const Material& m) {
    real metallic = clampf(m.parameters.y, K(0.0), K(1.0));
    real dielectric = dielectricF0(m.parameters2.y, m.parameters2.x);
    V3 dielectricColor = dielectric * clamp3(m.specularColor.xyz(), v3(K(0.0)), v3(K(1.0)));
    return mix3(dielectricColor, m.baseColor.xyz(), metallic);
}
static real materialClearcoat(const Material& m) { return clampf(m.parameters2.z, K(0.0), K(1.0)); }
static real materialClearcoatRoughness(const Material& m) { return clampf(m.parameters2.w, K(0.02), K(1.0)); }
static real materialClearcoatThickness(const Material& m) { return mx(m.clearcoatAttenuation.w, K(0.0)); }
static real materialClearcoatF0(const Material& m) { return dielectricF0(m.specularColor.w, K(1.0)); }
static V3 materialClearcoatF0Color(const Material& m) {
    return materialClearcoatF0(m) * clamp3(m.clearcoatColor.xyz(), v3(K(0.0)), v3(K(1.0)));
}
static V3 materialClearcoatAttenuationColor(const Material& m) {
    return clamp3(m.clearcoatAttenuation.xyz(), v3(K(0.0001)), v3(K(1.0)));
}
// materialClearcoatDepthAttenuation: PathTrace.metal:442-456
static V3 materialClearcoatDepthAttenuation(const Material& m, V3 normal, V3 view, V3 light) {
    real thickness = materialClearcoatThickness(m) * materialClearcoat(m);
    if (thickness <= K(1e-5)) return v3(K(1.0));
    real nDotV = mx(dot(normal, view), K(0.05));
    real nDotL = mx(dot(normal, light), K(0.05));
    real pathLength = thickness * K(0.5) * (K(1.0) / nDotV + K(1.0) / nDotL);
    return exp3(log3(materialClearcoatAttenuationColor(m)) * pathLength);
}
// Accessors: PathTrace.metal:458-548
static real materialSpecularAnisotropy(const Material& m) { return clampf(m.parameters3.w, K(-0.95), K(0.95)); }
static real materialTransmission(const Material& m) { return clampf(m.emission.w, K(0.0), K(1.0)); }
static V3 materialTransmissionColor(const Material& m) { return clamp3(m.transmissionColor.xyz(), v3(K(0.0)), v3(K(1.0))); }
static bool materialThinWalled(const Material& m) { return m.transmissionColor.w > K(0.5); }
static real materialTransmissionRoughness(const Material& m) { return clampf(m.parameters3.y, K(0.001), K(1.0)); }
static real materialTransmissionIOR(const Material& m) { return mx(m.parameters3.z, K(1.0001)); }
static real materialSheen(const Material& m) { return clampf(m.sheenColor.w, K(0.0), K(1.0)); }
static V3 materialSheenColor(const Material& m) { return clamp3(m.sheenColor.xyz(), v3(K(0.0)), v3(K(1.0))); }
static real materialSheenRoughness(const Material& m) { return clampf(m.parameters3.x, K(0.02), K(1.0)); }
static real materialSubsurface(const Material& m) {
    real metallic = clampf(m.parameters.y, K(0.0), K(1.0));
    real transmission = materialTransmission(m);
    return clampf(m.subsurfaceColor.w, K(0.0), K(1.0)) * (K(1.0) - metallic) * (K(1.0) - transmission);
}
static V3 materialSubsurfaceColor(const Material& m) { return clamp3(m.subsurfaceColor.xyz(), v3(K(0.0)), v3(K(0.999))); }
static V3 materialSubsurfaceRadius(const Material& m) {
    real scale = mx(m.subsurfaceRadius.w, K(0.0));
    return mx(m.subsurfaceRadius.xyz() * scale, v3(K(1e-4)));
}
static real materialSubsurfaceAnisotropy(const Material& m) { return clampf(m.subsurfaceParameters.x, K(-0.95), K(0.95)); }
static V3 materialTransmissionTint(const Material& m, real strength) {
    return mix3(v3(K(1.0)), materialTransmissionColor(m), strength);
}
static V3 materialTransmissionAbsorptionCoefficient(const Material& m) {
    real referenceDistance = m.transmissionAbsorption.w;
    if (referenceDistance <= K(1e-5)) return v3(K(0.0));
    V3 referenceColor = clamp3(m.transmissionAbsorption.xyz(), v3(K(0.0001)), v3(K(1.0)));
    return (-log3(referenceColor)) / referenceDistance;
}
static V3 materialTransmissionAbsorption(const Material& m, real distance, bool applies) {
    if (!applies || distance <= K(0.0)) return v3(K(1.0));
    return exp3((-materialTransmissionAbsorptionCoefficient(m)) * distance);
}
static real materialVolumeScattering(const Material& m) { return clampf(m.volumeScattering.w, K(0.0), K(1.0)); }
static V3 materialVolumeScatteringColor(const Material& m) { return clamp3(m.volumeScattering.xyz(), v3(K(0.0)), v3(K(1.0))); }
static real materialVolumeScatteringDistance(const Material& m) { return mx(m.volumeParameters.x, K(1e-4)); }
static real materialVolumeAnisotropy(const Material& m) { return clampf(m.volumeParameters.y, K(-0.95), K(0.95)); }
static bool materialHasVolumeScattering(const Material& m) {
    return materialTransmission(m) > K(0.0) && !materialThinWalled(m) && materialVolumeScattering(m) > K(0.0);
}
// blendMaterials: PathTrace.metal:527-547
static Material blendMaterials(Material a, const Material& b, real blend) {
    real t = clampf(blend, K(0.0), K(1.0));
    a.baseColor = mix4(a.baseColor, b.baseColor, t);
    a.emission = mix4(a.emission, b.emission, t);
    a.parameters = mix4(a.parameters, b.parameters, t);
    a.parameters2 = mix4(a.parameters2, b.parameters2, t);
    a.specularColor = mix4(a.specularColor, b.specularColor, t);
    a.sheenColor = mix4(a.sheenColor, b.sheenColor, t);
    a.transmissionColor = mix4(a.transmissionColor, b.transmissionColor, t);
    a.parameters3 = mix4(a.parameters3, b.parameters3, t);
    a.clearcoatColor = mix4(a.clearcoatColor, b.clearcoatColor, t);
    a.clearcoatAttenuation = mix4(a.clearcoatAttenuation, b.clearcoatAttenuation, t);
    a.transmissionAbsorption = mix4(a.transmissionAbsorption, b.transmissionAbsorption, t);
    a.thinFilm = mix4(a.thinFilm, b.thinFilm, t);
    a.subsurfaceColor = mix4(a.subsurfaceColor, b.subsurfaceColor, t);
    a.subsurfaceRadius = mix4(a.subsurfaceRadius, b.subsurfaceRadius, t);
    a.subsurfaceParameters = mix4(a.subsurfaceParameters, b.subsurfaceParameters, t);
    a.volumeScattering = mix4(a.volumeScattering, b.volumeScattering, t);
    a.volumeParameters = mix4(a.volumeParameters, b.volumeParameters, t);
    return a;
}
// materialForHit: PathTrace.metal:1096-1121.  The material-program VM and the
// volume field overrides are no-ops for triangle hits (no program, no flags).
static Material materialForHit(const Ctx& c, const Hit& hit) {
    count(c, C_MATERIAL_FETCH);
    uint32_t materialCount = c.s->material_count;
    uint32_t a = std::min(hit.materialID, materialCount - 1u);
    Material m = loadMaterial(c.s->materials[a]);
    if (hit.materialBlend > K(0.0)) {
        uint32_t b = std::min(hit.materialID2, materialCount - 1u);
        m = blendMaterials(m, loadMaterial(c.s->materials[b]), hit.materialBlend);
    }
    return m;
}
// materialVolumeSigmaS / SigmaT / Transmittance: PathTrace.metal:1137-1150
static V3 materialVolumeSigmaS(const Material& m) {
    return materialVolumeScatteringColor(m) * materialVolumeScattering(m) / materialVolumeScatteringDistance(m);
}
static V3 materialVolumeSigmaT(const Material& m) {
    return materialTransmissionAbsorptionCoefficient(m) + materialVolumeSigmaS(m);
}
static V3 materialVolumeTransmittance(const Material& m, real distance) {
    return exp3((-materialVolumeSigmaT(m)) * distance);
}

// makeTangentFrame: PathTrace.metal:1157-1176
struct TangentFrame { V3 tangent, bitangent; };
static TangentFrame makeTangentFrame(V3 normal, V3 rawTangent, V3 rawBitangent) {
    TangentFrame f;
    V3 tangent = rawTangent - normal * dot(rawTangent, normal);
    if (dot(tangent, tangent) <= K(1e-8)) {
        V3 helper = std::fabs(normal.y) < K(0.999) ? v3(0, 1, 0) : v3(1, 0, 0);
        tangent = cross(helper, normal);
    }
    f.tangent = normalize(tangent);
    V3 bitangent = rawBitangent - normal * dot(rawBitangent, normal) - f.tangent * dot(rawBitangent, f.tangent);
    if (dot(bitangent, bitangent) <= K(1e-8)) bitangent = cross(normal, f.tangent);
    f.bitangent = normalize(bitangent);
    return f;
}
// anisotropicGGXAlpha: PathTrace.metal:1178-1187
static V2 anisotropicGGXAlpha(real roughness, real anisotropy) {
    real alpha = mx(roughness * roughness, K(0.001));
    real amount = clampf(anisotropy, K(-0.95), K(0.95));
    real aspect = std::sqrt(mx(K(0.1), K(1.0) - K(0.9) * std::fabs(amount)));
    real alphaLong = alpha / aspect;
    real alphaShort = alpha * aspect;
    return amount >= K(0.0) ? v2(alphaLong, alphaShort) : v2(alphaShort, alphaLong);
}
// distributionGGX / geometrySmithG1GGX / geometrySmith: PathTrace.metal:1189-1205
static real distributionGGX(real nDotH, real roughness) {
    real alpha = roughness * roughness;
    real alpha2 = alpha * alpha;
    real denominator = nDotH * nDotH * (alpha2 - K(1.0)) + K(1.0);
    return alpha2 / mx(K(3.14159265359) * denominator * denominator, K(1e-5));
}
static real geometrySmithG1GGX(real nDotV, real roughness) {
    real alpha = roughness * roughness;
    real alpha2 = alpha * alpha;
    real denominator = nDotV + std::sqrt(mx(alpha2 + (K(1.0) - alpha2) * nDotV * nDotV, K(0.0)));
    return (K(2.0) * nDotV) / mx(denominator, K(1e-5));
}
static real geometrySmith(real nDotV, real nDotL, real roughness) {
    return geometrySmithG1GGX(nDotV, roughness) * geometrySmithG1GGX(nDotL, roughness);
}
// distributionGGXAnisotropic: PathTrace.metal:1207-1227
static real distributionGGXAnisotropic(V3 h, V3 n, V3 t, V3 b, real roughness, real anisotropy) {
    real nDotH = mx(dot(n, h), K(0.0));
    if (nDotH <= K(0.0)) return K(0.0);
    V2 alpha = anisotropicGGXAlpha(roughness, anisotropy);
    real tDotH = dot(t, h);
    real bDotH = dot(b, h);
    real denominator = (tDotH * tDotH) / mx(alpha.x * alpha.x, K(1e-6)) + (bDotH * bDotH) / mx(alpha.y * alpha.y, K(1e-6)) + nDotH * nDotH;
    return K(1.0) / mx(K(3.14159265359) * alpha.x * alpha.y * denominator * denominator, K(1e-6));
}
// geometrySmithG1GGXAnisotropic / geometrySmithAnisotropic: PathTrace.metal:1229-1264
static real geometrySmithG1GGXAnisotropic(V3 d, V3 n, V3 t, V3 b, real roughness, real anisotropy) {
    real nDotD = mx(dot(n, d), K(0.0));
    if (nDotD <= K(0.0)) return K(0.0);
    V2 alpha = anisotropicGGXAlpha(roughness, anisotropy);
    real tDotD = dot(t, d);
    real bDotD = dot(b, d);
    real root = std::sqrt(mx(alpha.x * alpha.x * tDotD * tDotD + alpha.y * alpha.y * bDotD * bDotD + nDotD * nDotD, K(0.0)));
    return (K(2.0) * nDotD) / mx(nDotD + root, K(1e-5));
}
static real geometrySmithAnisotropic(V3 v, V3 l, V3 n, V3 t, V3 b, real roughness, real anisotropy) {
    return geometrySmithG1GGXAnisotropic(v, n, t, b, roughness, anisotropy) *
           geometrySmithG1GGXAnisotropic(l, n, t, b, roughness, anisotropy);
}
// evaluateMaterialSheenBRDF: PathTrace.metal:1266-1297
static V3 evaluateMaterialSheenBRDF(const Material& m, V3 normal, V3 view, V3 light) {
    real sheen = materialSheen(m);
    if (sheen <= K(0.0)) return v3(K(0.0));
    real metallic = clampf(m.parameters.y, K(0.0), K(1.0));
    V3 halfDirection = view + light;
    if (dot(halfDirection, halfDirection) <= K(1e-8)) return v3(K(0.0));
    V3 halfVector = normalize(halfDirection);
    real nDotL = mx(dot(normal, light), K(0.0));
    real nDotV = mx(dot(normal, view), K(0.0));
    real nDotH = mx(dot(normal, halfVector), K(0.0));
    if (nDotL <= K(0.0) || nDotV <= K(0.0)) return v3(K(0.0));
    real sinThetaH = std::sqrt(mx(K(0.0), K(1.0) - nDotH * nDotH));
    real inverseAlpha = mixf(K(20.0), K(0.5), materialSheenRoughness(m));
    real distribution = (K(2.0) + inverseAlpha) * std::pow(sinThetaH, inverseAlpha) * K(0.15915494309);
    real visibility = K(1.0) / mx(K(4.0) * (nDotL + nDotV - nDotL * nDotV), K(1e-5));
    return sheen * (K(1.0) - metallic) * materialSheenColor(m) * distribution * visibility;
}
// materialClearcoatAttenuationForDirection: PathTrace.metal:1299-1321
static V3 materialClearcoatAttenuationForDirection(const Material& m, V3 normal, V3 view, V3 light) {
    real clearcoat = materialClearcoat(m);
    if (clearcoat <= K(0.0)) return v3(K(1.0));
    V3 halfDirection = view + light;
    if (dot(halfDirection, halfDirection) <= K(1e-8)) return v3(K(1.0));
    V3 halfVector = normalize(halfDirection);
    real vDotH = mx(dot(view, halfVector), K(0.0));
    V3 clearcoatFresnel = fresnelSchlickThinFilm(vDotH, materialClearcoatF0Color(m), m);
    V3 fresnelAttenuation = mx(v3(K(0.0)), v3(K(1.0)) - clearcoatFresnel * clearcoat);
    return fresnelAttenuation * materialClearcoatDepthAttenuation(m, normal, view, light);
}
// evaluateMaterialBRDF: PathTrace.metal:1323-1384
static V3 evaluateMaterialBRDF(const Material& m, V3 normal, V3 tangent, V3 bitangent, V3 view, V3 light) {
    const real inversePi = K(0.31830988618);
    real roughness = clampf(m.parameters.x, K(0.02), K(1.0));
    real metallic = clampf(m.parameters.y, K(0.0), K(1.0));
    V3 baseColor = m.baseColor.xyz();
    V3 halfVector = normalize(view + light);
    real nDotL = mx(dot(normal, light), K(0.0));
    real nDotV = mx(dot(normal, view), K(0.0));
    real nDotH = mx(dot(normal, halfVector), K(0.0));
    real vDotH = mx(dot(view, halfVector), K(0.0));
    if (nDotL <= K(0.0) || nDotV <= K(0.0)) return v3(K(0.0));
    V3 f0 = materialF0(m);
    V3 fresnel = fresnelSchlickThinFilm(vDotH, f0, m);
    TangentFrame frame = makeTangentFrame(normal, tangent, bitangent);
    real anisotropy = materialSpecularAnisotropy(m);
    real distribution = distributionGGXAnisotropic(halfVector, normal, frame.tangent, frame.bitangent, roughness, anisotropy);
    real geometry = geometrySmithAnisotropic(view, light, normal, frame.tangent, frame.bitangent, roughness, anisotropy);
    V3 specular = distribution * geometry * fresnel / mx(K(4.0) * nDotV * nDotL, K(1e-5));
    real clearcoat = materialClearcoat(m);
    real clearcoatRoughness = materialClearcoatRoughness(m);
    V3 clearcoatFresnel = fresnelSchlickThinFilm(vDotH, materialClearcoatF0Color(m), m);
    real clearcoatDistribution = distributionGGX(nDotH, clearcoatRoughness);
    real clearcoatGeometry = geometrySmith(nDotV, nDotL, clearcoatRoughness);
    V3 clearcoatSpecular = clearcoatDistribution * clearcoatGeometry * clearcoatFresnel / mx(K(4.0) * nDotV * nDotL, K(1e-5));
    V3 clearcoatAttenuation = materialClearcoatAttenuationForDirection(m, normal, view, light);
    V3 diffuse = clearcoatAttenuation * (v3(K(1.0)) - fresnel) * (K(1.0) - metallic) * baseColor * inversePi;
    V3 sheen = evaluateMaterialSheenBRDF(m, normal, view, light);
    return diffuse + clearcoatAttenuation * (specular + sheen) + clearcoatSpecular * clearcoat;
}
// powerHeuristic: PathTrace.metal:1386-1390
static real powerHeuristic(real a, real b) {
    real a2 = a * a;
    real b2 = b * b;
    return a2 / mx(a2 + b2, K(1e-8));
}
// materialLobeProbabilities: PathTrace.metal:1392-1422
static void materialLobeProbabilities(const Material& m, real& diffuseP, real& specularP, real& clearcoatP) {
    real metallic = clampf(m.parameters.y, K(0.0), K(1.0));
    V3 baseColor = m.baseColor.xyz();
    V3 f0 = materialF0(m);
    real clearcoat = materialClearcoat(m);
    real sheenWeight = materialSheen(m) * luminance(materialSheenColor(m)) * (K(1.0) - metallic);
    real diffuseWeight = luminance(baseColor * (K(1.0) - metallic)) + sheenWeight;
    real specularWeight = luminance(f0);
    real clearcoatWeight = clearcoat * luminance(materialClearcoatF0Color(m));
    real totalLobeWeight = mx(diffuseWeight + specularWeight + clearcoatWeight, K(1e-5));
    clearcoatP = clearcoatWeight > K(1e-5) ? clampf(clearcoatWeight / totalLobeWeight, K(0.02), K(0.35)) : K(0.0);
    real remaining = mx(K(0.0), K(1.0) - clearcoatP);
    if (specularWeight <= K(1e-5)) {
        specularP = K(0.0);
    } else if (diffuseWeight <= K(1e-5)) {
        specularP = remaining;
    } else {
        specularP = clampf(specularWeight / totalLobeWeight, K(0.08), remaining);
    }
    diffuseP = mx(K(0.0), K(1.0) - specularP - clearcoatP);
}
// ggxReflectionPDF: PathTrace.metal:1424-1443
static real ggxReflectionPDF(V3 n, V3 t, V3 b, V3 view, V3 light, real roughness, real anisotropy) {
    V3 h = normalize(view + light);
    real nDotH = mx(dot(n, h), K(0.0));
    real nDotV = mx(dot(n, view), K(0.0));
    real vDotH = mx(dot(view, h), K(0.0));
    if (nDotH <= K(0.0) || nDotV <= K(0.0) || vDotH <= K(0.0)) return K(0.0);
    TangentFrame f = makeTangentFrame(n, t, b);
    return distributionGGXAnisotropic(h, n, f.tangent, f.bitangent, roughness, anisotropy) *
           geometrySmithG1GGXAnisotropic(view, n, f.tangent, f.bitangent, roughness, anisotropy) / mx(K(4.0) * nDotV, K(1e-5));
}
// materialBSDFPDF: PathTrace.metal:1445-1490
static real materialBSDFPDF(const Material& m, V3 n, V3 t, V3 b, V3 view, V3 light) {
    const real inversePi = K(0.31830988618);
    real nDotL = mx(dot(n, light), K(0.0));
    real nDotV = mx(dot(n, view), K(0.0));
    if (nDotL <= K(0.0) || nDotV <= K(0.0)) return K(0.0);
    real dP, sP, cP;
    materialLobeProbabilities(m, dP, sP, cP);
    real roughness = clampf(m.parameters.x, K(0.02), K(1.0));
    real clearcoatRoughness = materialClearcoatRoughness(m);
    real anisotropy = materialSpecularAnisotropy(m);
    real diffusePDF = nDotL * inversePi;
    real specularPDF = ggxReflectionPDF(n, t, b, view, light, roughness, anisotropy);
    real clearcoatPDF = ggxReflectionPDF(n, t, b, view, light, clearcoatRoughness, K(0.0));
    return dP * diffusePDF + sP * specularPDF + cP * clearcoatPDF;
}
// materialDiffuseBounceWeight: PathTrace.metal:1492-1518
static V3 materialDiffuseBounceWeight(const Material& m, V3 normal, V3 view, V3 light) {
    real metallic = clampf(m.parameters.y, K(0.0), K(1.0));
    V3 baseColor = m.baseColor.xyz();
    V3 halfDirection = view + light;
    if (dot(halfDirection, halfDirection) <= K(1e-8)) return v3(K(0.0));
    V3 halfVector = normalize(halfDirection);
    real vDotH = mx(dot(view, halfVector), K(0.0));
    V3 fresnel = fresnelSchlickThinFilm(vDotH, materialF0(m), m);
    V3 clearcoatAttenuation = materialClearcoatAttenuationForDirection(m, normal, view, light);
    V3 diffuse = (v3(K(1.0)) - fresnel) * (K(1.0) - metallic) * baseColor;
    V3 sheen = evaluateMaterialSheenBRDF(m, normal, view, light) * K(3.14159265359);
    return clearcoatAttenuation * (diffuse + sheen);
}
// terminatePathWithRussianRoulette: PathTrace.metal:1520-1540
static bool terminatePathWithRussianRoulette(uint32_t bounce, V3& throughput, uint32_t& state) {
    real continuationWeight = maxComponent(throughput);
    if (continuationWeight <= K(0.0)) return true;
    if (bounce < 2u) return false;
    real survival = clampf(continuationWeight, K(0.05), K(0.95));
    if (randomFloat(state) > survival) return true;
    throughput /= survival;
    return false;
}

// ------------------------------------------------------------- lights -----
// lightSolidAnglePDF / lightSelectionCDF / lightSelectionPDF: PathTrace.metal:1542-1557
static real lightSolidAnglePDF(real distanceSquared, real cosLight, real area) {
    return distanceSquared / mx(cosLight * area, K(1e-6));
}
static real lightSelectionCDF(const Ctx& c, uint32_t i) { return clampf((real)c.s->lights[i].selection_cdf, K(0.0), K(1.0)); }
static real lightSelectionPDF(const Ctx& c, uint32_t i) {
    real previous = i == 0u ? K(0.0) : lightSelectionCDF(c, i - 1u);
    return mx(lightSelectionCDF(c, i) - previous, K(0.0));
}
// selectLightIndex: PathTrace.metal:1559-1576
static uint32_t selectLightIndex(const Ctx& c, uint32_t lightCount, real sample) {
    if (lightCount <= 1u) return 0u;
    real target = clampf(sample, K(0.0), (real)0.99999994f);
    uint32_t low = 0u, high = lightCount - 1u;
    while (low < high) {
        uint32_t mid = (low + high) >> 1u;
        if (target <= lightSelectionCDF(c, mid)) high = mid; else low = mid + 1u;
    }
    return low;
}
// lightPDFForHit: PathTrace.metal:1578-1608
static real lightPDFForHit(const Ctx& c, const Hit& hit, V3 incoming) {
    if (hit.primitiveID >= c.s->triangle_count) return K(0.0);
    uint32_t plus1 = c.s->triangles[hit.primitiveID].padding2;
    if (plus1 == 0u) return K(0.0);
    uint32_t index = plus1 - 1u;
    if (index >= c.s->light_count) return K(0.0);
    const dk_light_record& light = c.s->lights[index];
    if (light.triangle_index != hit.primitiveID || (real)light.area <= K(0.0)) return K(0.0);
    real cosLight = mx(K(0.0), dot(ld3(light.normal), -incoming));
    if (cosLight <= K(0.0)) return K(0.0);
    return lightSelectionPDF(c, index) * lightSolidAnglePDF(hit.t * hit.t, cosLight, (real)light.area);
}
// sampleGGXHalfVector: PathTrace.metal:1610-1618
static V3 sampleGGXHalfVector(V2 u, V3 normal, real roughness) {
    real alpha = roughness * roughness;
    real alpha2 = alpha * alpha;
    real phi = K(6.28318530718) * u.x;
    real cosTheta = std::sqrt((K(1.0) - u.y) / mx(K(1.0) + (alpha2 - K(1.0)) * u.y, K(1e-5)));
    real sinTheta = std::sqrt(mx(K(0.0), K(1.0) - cosTheta * cosTheta));
    V3 local = v3(std::cos(phi) * sinTheta, std::sin(phi) * sinTheta, cosTheta);
    return orientHemisphere(local, normal);
}
// sampleGGXVisibleNormal: PathTrace.metal:1620-1660
static V3 sampleGGXVisibleNormal(V2 u, V3 normal, V3 tangent, V3 bitangent, V3 view, real roughness, real anisotropy) {
    TangentFrame frame = makeTangentFrame(normal, tangent, bitangent);
    V2 alpha = anisotropicGGXAlpha(roughness, anisotropy);
    V3 localView = normalize(v3(dot(view, frame.tangent), dot(view, frame.bitangent), mx(dot(view, normal), K(1e-5))));
    V3 stretchedView = normalize(v3(alpha.x * localView.x, alpha.y * localView.y, localView.z));
    real lensq = stretchedView.x * stretchedView.x + stretchedView.y * stretchedView.y;
    V3 t1 = lensq > K(1e-7) ? v3(-stretchedView.y, stretchedView.x, K(0.0)) * (K(1.0) / std::sqrt(lensq)) : v3(1, 0, 0);
    V3 t2 = cross(stretchedView, t1);
    real radius = std::sqrt(u.x);
    real phi = K(6.28318530718) * u.y;
    real p1 = radius * std::cos(phi);
    real p2 = radius * std::sin(phi);
    real blend = K(0.5) * (K(1.0) + stretchedView.z);
    p2 = mixf(std::sqrt(mx(K(0.0), K(1.0) - p1 * p1)), p2, blend);
    V3 visibleNormal = p1 * t1 + p2 * t2 + std::sqrt(mx(K(0.0), K(1.0) - p1 * p1 - p2 * p2)) * stretchedView;
    V3 localHalf = normalize(v3(alpha.x * visibleNormal.x, alpha.y * visibleNormal.y, mx(visibleNormal.z, K(0.0))));
    return normalize(localHalf.x * frame.tangent + localHalf.y * frame.bitangent + localHalf.z * normal);
}
// projectToScreen: PathTrace.metal:1662-1697
static bool projectToScreen(const dk_camera& cam, V3 world, uint32_t width, uint32_t height, V2& screen) {
    V3 horizontal = ld3(cam.horizontal), vertical = ld3(cam.vertical), lowerLeft = ld3(cam.lower_left), origin = ld3(cam.origin);
    V3 forward = normalize(cross(vertical, horizontal));
    V3 planeCenter = lowerLeft + horizontal * K(0.5) + vertical * K(0.5);
    V3 planePoint;
    if ((real)cam.origin.w > K(0.5)) {
        planePoint = world - forward * dot(world - planeCenter, forward);
    } else {
        V3 toPoint = world - origin;
        real denominator = dot(toPoint, forward);
        if (std::fabs(denominator) <= K(1e-5)) return false;
        real planeDistance = dot(planeCenter - origin, forward);
        real planeT = planeDistance / denominator;
        if (planeT <= K(0.0)) return false;
        planePoint = origin + toPoint * planeT;
    }
    V3 relative = planePoint - lowerLeft;
    real u = dot(relative, horizontal) / mx(dot(horizontal, horizontal), K(1e-5));
    real v = dot(relative, vertical) / mx(dot(vertical, vertical), K(1e-5));
    screen = v2(u * (real)width, (K(1.0) - v) * (real)height);
    return true;
}
// sampleTriangle: PathTrace.metal:1711-1717
static V3 sampleTriangle(const dk_triangle& tri, V2 r) {
    real su0 = std::sqrt(r.x);
    real b0 = K(1.0) - su0;
    real b1 = su0 * (K(1.0) - r.y);
    real b2 = su0 * r.y;
    return b0 * ld3(tri.v0) + b1 * ld3(tri.v1) + b2 * ld3(tri.v2);
}

// ------------------------------------------------------- intersection -----
// intersectTriangle (Möller-Trumbore): PathTrace.metal:1801-1852
static bool intersectTriangle(const Ray& ray, const dk_triangle& tri, real& t, V3& normal, V2& uv, V3& tangent,
                              V3& bitangent, bool& frontFacing) {
    V3 p0 = ld3(tri.v0), p1 = ld3(tri.v1), p2 = ld3(tri.v2);
    V3 edge1 = p1 - p0;
    V3 edge2 = p2 - p0;
    V3 p = cross(ray.direction, edge2);
    real determinant = dot(edge1, p);
    if (std::fabs(determinant) < K(1e-7)) return false;
    real invDeterminant = K(1.0) / determinant;
    V3 s = ray.origin - p0;
    real u = invDeterminant * dot(s, p);
    if (u < K(0.0) || u > K(1.0)) return false;
    V3 q = cross(s, edge1);
    real v = invDeterminant * dot(ray.direction, q);
    if (v < K(0.0) || u + v > K(1.0)) return false;
    real candidateT = invDeterminant * dot(edge2, q);
    if (candidateT <= K(0.0005)) return false;
    t = candidateT;
    real w = K(1.0) - u - v;
    normal = normalize(w * ld3(tri.n0) + u * ld3(tri.n1) + v * ld3(tri.n2));
    frontFacing = dot(normal, ray.direction) <= K(0.0);
    if (dot(normal, ray.direction) > K(0.0)) normal = -normal;
    uv = w * v2((real)tri.uv0.x, (real)tri.uv0.y) + u * v2((real)tri.uv1.x, (real)tri.uv1.y) + v * v2((real)tri.uv2.x, (real)tri.uv2.y);
    tangent = normalize(ld3(tri.tangent));
    bitangent = normalize(ld3(tri.bitangent));
    return true;
}
// intersectBounds: PathTrace.metal:1854-1863
static bool intersectBounds(const Ray& ray, const dk_bvh_node& node, real closestT) {
    V3 invDirection = K(1.0) / ray.direction;
    V3 t0 = (ld3(node.bounds_min) - ray.origin) * invDirection;
    V3 t1 = (ld3(node.bounds_max) - ray.origin) * invDirection;
    V3 tNear3 = mn(t0, t1);
    V3 tFar3 = mx(t0, t1);
    real tNear = mx(mx(tNear3.x, tNear3.y), mx(tNear3.z, K(0.0)));
    real tFar = mn(mn(tFar3.x, tFar3.y), mn(tFar3.z, closestT));
    return tNear <= tFar;
}
// emptyHit: PathTrace.metal:1883-1909
static Hit emptyHit() {
    Hit h;
    h.hit = false;
    h.t = (real)INFINITY;
    h.position = v3(K(0.0));
    h.normal = v3(0, 1, 0);
    h.uv = v2(0, 0);
    h.tangent = v3(1, 0, 0);
    h.bitangent = v3(0, 0, 1);
    h.materialID = 0;
    h.materialID2 = 0;
    h.materialBlend = K(0.0);
    h.objectID = 0;
    h.primitiveID = 0;
    h.frontFacing = true;
    return h;
}
static void recordHit(Hit& closest, const Ray& ray, const dk_triangle& tri, uint32_t triangleIndex, real t, V3 normal,
                      V2 uv, V3 tangent, V3 bitangent, bool frontFacing) {
    closest.hit = true;
    closest.t = t;
    closest.position = ray.origin + t * ray.direction;
    closest.normal = normal;
    closest.uv = uv;
    closest.tangent = tangent;
    closest.bitangent = bitangent;
    closest.materialID = tri.material_id;
    closest.materialID2 = tri.material_id;
    closest.materialBlend = K(0.0);
    closest.objectID = tri.object_id;
    closest.primitiveID = triangleIndex;
    closest.frontFacing = frontFacing;
}
#include "sparse_oracle.inc"

// intersectSceneLinear / intersectScene: PathTrace.metal:3264-3421 (binary BVH,
// 64-entry stack, left child first, strict `t < closest.t`).
static Hit intersectScene(const Ctx& c, const Ray& ray, int kind) {
    count(c, C_QUERIES_K0 + kind);
    Hit closest = emptyHit();
    const dk_scene* s = c.s;
    if (s->node_count == 0 || s->nodes == nullptr || s->primitive_indices == nullptr) {
        for (uint32_t i = 0; i < s->triangle_count; ++i) {
            real t; V3 n; V2 uv; V3 tg, bt; bool ff;
            count(c, C_TRIS_K0 + kind);
            if (intersectTriangle(ray, s->triangles[i], t, n, uv, tg, bt, ff) && t < closest.t)
                recordHit(closest, ray, s->triangles[i], i, t, n, uv, tg, bt, ff);
        }
        Hit vh = closestVolumeHit(c, ray, closest.t);
        return vh.hit ? vh : closest;
    }
    uint32_t stack[64];
    uint32_t stackCount = 0;
    stack[stackCount++] = 0;
    while (stackCount > 0) {
        uint32_t nodeIndex = stack[--stackCount];
        if (nodeIndex >= s->node_count) continue;
        const dk_bvh_node& node = s->nodes[nodeIndex];
        count(c, C_NODES_K0 + kind);
        if (!intersectBounds(ray, node, closest.t)) continue;
        uint32_t first = node.metadata.z, primCount = node.metadata.w;
        if (primCount > 0) {
            for (uint32_t o = 0; o < primCount; ++o) {
                uint32_t ti = s->primitive_indices[first + o];
                if (ti >= s->triangle_count) continue;
                real t; V3 n; V2 uv; V3 tg, bt; bool ff;
                count(c, C_TRIS_K0 + kind);
                if (intersectTriangle(ray, s->triangles[ti], t, n, uv, tg, bt, ff) && t < closest.t)
                    recordHit(closest, ray, s->triangles[ti], ti, t, n, uv, tg, bt, ff);
            }
        } else if (stackCount + 2u <= 64u) {
            stack[stackCount++] = node.metadata.y;
            stack[stackCount++] = node.metadata.x;
        }
    }
    Hit vh = closestVolumeHit(c, ray, closest.t);
    if (vh.hit) closest = vh;
    return closest;
}

// ---------------------------------------------------- random walks --------
// Subsurface helpers: PathTrace.metal:3490-3523
static V3 subsurfaceSigmaT(const Material& m) { return K(1.0) / materialSubsurfaceRadius(m); }
static real sampleSubsurfaceFreeFlight(V3 sigmaT, V2 u) {
    real sigma = sigmaT.z;
    if (u.x < K(0.33333333333)) sigma = sigmaT.x;
    else if (u.x < K(0.66666666667)) sigma = sigmaT.y;
    return -std::log(mx(K(1.0) - u.y, K(1e-6))) / mx(sigma, K(1e-4));
}
static real subsurfaceCollisionPDF(V3 sigmaT, real d) {
    V3 tr = exp3((-sigmaT) * d);
    return mx((sigmaT.x * tr.x + sigmaT.y * tr.y + sigmaT.z * tr.z) * K(0.33333333333), K(1e-6));
}
static real subsurfaceBoundaryPDF(V3 sigmaT, real d) {
    V3 tr = exp3((-sigmaT) * d);
    return mx((tr.x + tr.y + tr.z) * K(0.33333333333), K(1e-6));
}
static V3 subsurfaceCollisionWeight(V3 sigmaT, V3 albedo, real d) {
    V3 tr = exp3((-sigmaT) * d);
    return albedo * sigmaT * tr / subsurfaceCollisionPDF(sigmaT, d);
}
static V3 subsurfaceBoundaryWeight(V3 sigmaT, real d) {
    V3 tr = exp3((-sigmaT) * d);
    return tr / subsurfaceBoundaryPDF(sigmaT, d);
}
// continueSubsurfaceRandomWalk: PathTrace.metal:3525-3621
static bool continueSubsurfaceRandomWalk(const Ctx& c, const Hit& entry, const Material& m, Ray& ray, V3& throughput,
                                         real& previousPDF, uint32_t& state) {
    real subsurface = materialSubsurface(m);
    if (subsurface <= K(0.0) || !entry.frontFacing) return false;
    real e0 = randomFloat(state);
    real e1 = randomFloat(state);
    V3 entryDirection = orientHemisphere(cosineHemisphere(v2(e0, e1)), -entry.normal);
    Ray medium;
    medium.origin = entry.position + entryDirection * K(0.001);
    medium.direction = entryDirection;
    V3 sigmaT = subsurfaceSigmaT(m);
    V3 albedo = materialSubsurfaceColor(m);
    real anisotropy = materialSubsurfaceAnisotropy(m);
    for (uint32_t step = 0u; step < 8u; ++step) {
        Hit boundary = intersectScene(c, medium, 2);
        if (!boundary.hit) return false;
        real f0 = randomFloat(state);
        real f1 = randomFloat(state);
        real freeFlight = sampleSubsurfaceFreeFlight(sigmaT, v2(f0, f1));
        if (freeFlight < boundary.t) {
            medium.origin += medium.direction * freeFlight;
            real h0 = randomFloat(state);
            real h1 = randomFloat(state);
            medium.direction = sampleHenyeyGreenstein(v2(h0, h1), medium.direction, anisotropy);
            throughput *= subsurfaceCollisionWeight(sigmaT, albedo, freeFlight);
            if (maxComponent(throughput) <= K(1e-4)) return false;
            continue;
        }
        V3 exitNormal = boundary.frontFacing ? boundary.normal : -boundary.normal;
        exitNormal = normalize(exitNormal);
        real x0 = randomFloat(state);
        real x1 = randomFloat(state);
        V3 local = cosineHemisphere(v2(x0, x1));
        ray.direction = orientHemisphere(local, exitNormal);
        ray.origin = boundary.position + exitNormal * K(0.001);
        throughput *= subsurfaceBoundaryWeight(sigmaT, boundary.t);
        previousPDF = mx(dot(exitNormal, ray.direction), K(0.0)) * K(0.31830988618);
        return true;
    }
    return false;
}
// continueTransmissionVolumeRandomWalk: PathTrace.metal:3685-3721
static bool continueTransmissionVolumeRandomWalk(const Hit& boundary, const Material& m, Ray& ray, V3& throughput,
                                                 real& previousPDF, uint32_t& state) {
    if (boundary.frontFacing || !materialHasVolumeScattering(m)) return false;
    V3 sigmaT = materialVolumeSigmaT(m);
    V3 sigmaS = materialVolumeSigmaS(m);
    if (maxComponent(sigmaT) <= K(1e-5) || maxComponent(sigmaS) <= K(1e-5)) return false;
    real f0 = randomFloat(state);
    real f1 = randomFloat(state);
    real freeFlight = sampleSubsurfaceFreeFlight(sigmaT, v2(f0, f1));
    if (freeFlight >= boundary.t) {
        throughput *= materialVolumeTransmittance(m, boundary.t) / subsurfaceBoundaryPDF(sigmaT, boundary.t);
        return false;
    }
    V3 transmittance = exp3((-sigmaT) * freeFlight);
    throughput *= sigmaS * transmittance / subsurfaceCollisionPDF(sigmaT, freeFlight);
    ray.origin += ray.direction * freeFlight;
    real h0 = randomFloat(state);
    real h1 = randomFloat(state);
    ray.direction = sampleHenyeyGreenstein(v2(h0, h1), ray.direction, materialVolumeAnisotropy(m));
    ray.origin += ray.direction * K(0.001);
    previousPDF = K(0.0);
    return maxComponent(throughput) > K(1e-4);
}
// continueTransmissiveSurface: PathTrace.metal:1723-1799
static bool continueTransmissiveSurface(const Hit& hit, const Material& m, Ray& ray, V3& throughput,
                                        real& previousPDF, uint32_t& state) {
    real transmission = materialTransmission(m);
    if (transmission <= K(0.0) || randomFloat(state) > transmission) return false;
    V3 incoming = ray.direction;
    V3 view = -incoming;
    real roughness = materialTransmissionRoughness(m);
    real ior = materialTransmissionIOR(m);
    V3 microNormal = hit.normal;
    if (roughness > K(0.01)) {
        real a = randomFloat(state);
        real b = randomFloat(state);
        microNormal = sampleGGXHalfVector(v2(a, b), hit.normal, roughness);
        if (dot(microNormal, incoming) > K(0.0)) microNormal = -microNormal;
    }
    real etaI = hit.frontFacing ? K(1.0) : ior;
    real etaT = hit.frontFacing ? ior : K(1.0);
    real eta = etaI / etaT;
    real cosThetaI = mx(dot(view, microNormal), K(0.0));
    real fresnel = dielectricFresnel(cosThetaI, etaI, etaT);
    if (materialThinWalled(m)) {
        fresnel = dielectricFresnel(cosThetaI, K(1.0), ior);
        real reflectP = clampf(fresnel, K(0.02), K(0.98));
        if (randomFloat(state) < reflectP) {
            ray.direction = normalize(reflect(incoming, microNormal));
            ray.origin = hit.position + microNormal * K(0.001);
            throughput *= fresnel / mx(reflectP, K(1e-5));
        } else {
            ray.direction = incoming;
            ray.origin = hit.position + ray.direction * K(0.001);
            real grazing = K(1.0) - std::fabs(dot(view, hit.normal));
            real tintStrength = mixf(K(0.35), K(0.95), grazing * grazing);
            real transmissionWeight = (K(1.0) - fresnel) / mx(K(1.0) - reflectP, K(1e-5));
            throughput *= materialTransmissionTint(m, tintStrength) * transmissionWeight;
        }
        previousPDF = K(0.0);
        return true;
    }
    V3 refracted = refract(incoming, microNormal, eta);
    bool tir = dot(refracted, refracted) <= K(1e-7);
    real reflectP = tir ? K(1.0) : clampf(fresnel, K(0.02), K(0.98));
    if (randomFloat(state) < reflectP) {
        ray.direction = normalize(reflect(incoming, microNormal));
        ray.origin = hit.position + microNormal * K(0.001);
        throughput *= tir ? K(1.0) : fresnel / mx(reflectP, K(1e-5));
    } else {
        ray.direction = normalize(refracted);
        ray.origin = hit.position + ray.direction * K(0.001);
        real grazing = K(1.0) - std::fabs(dot(view, hit.normal));
        real tintStrength = mixf(K(0.35), K(0.95), grazing * grazing);
        real transmissionWeight = (K(1.0) - fresnel) / mx(K(1.0) - reflectP, K(1e-5));
        V3 absorption = materialTransmissionAbsorption(m, hit.t, !hit.frontFacing && !materialHasVolumeScattering(m));
        throughput *= materialTransmissionTint(m, tintStrength) * absorption * transmissionWeight;
    }
    previousPDF = K(0.0);
    return true;
}

// ------------------------------------------- textures and environment -----
// sampleTexture: PathTrace.metal:3723-3763
static V4 sampleTexture(const Ctx& c, uint32_t indexPlusOne, V2 uv, V4 fallback) {
    const dk_scene* s = c.s;
    if (indexPlusOne == 0u || s->texture_descriptors == nullptr || s->texture_pixels == nullptr) return fallback;
    const dk_texture_descriptor& d = s->texture_descriptors[indexPlusOne - 1u];
    uint32_t offset = d.metadata.x, width = d.metadata.y, height = d.metadata.z, mode = d.metadata.w;
    if (width == 0u || height == 0u) return fallback;
    V2 wrapped = v2(fractf(uv.x), fractf(uv.y));
    if (mode == 1u && width > 1u && height > 1u) {
        V2 tp = v2(wrapped.x * (real)width - K(0.5), wrapped.y * (real)height - K(0.5));
        V2 base = v2(std::floor(tp.x), std::floor(tp.y));
        V2 blend = v2(fractf(tp.x), fractf(tp.y));
        uint32_t x0 = (uint32_t)std::fmod(base.x + (real)width, (real)width);
        uint32_t y0 = (uint32_t)std::fmod(base.y + (real)height, (real)height);
        uint32_t x1 = (x0 + 1u) % width;
        uint32_t y1 = (y0 + 1u) % height;
        V4 c00 = ld4(s->texture_pixels[offset + y0 * width + x0]);
        V4 c10 = ld4(s->texture_pixels[offset + y0 * width + x1]);
        V4 c01 = ld4(s->texture_pixels[offset + y1 * width + x0]);
        V4 c11 = ld4(s->texture_pixels[offset + y1 * width + x1]);
        return mix4(mix4(c00, c10, blend.x), mix4(c01, c11, blend.x), blend.y);
    }
    uint32_t x = std::min((uint32_t)(wrapped.x * (real)width), width - 1u);
    uint32_t y = std::min((uint32_t)(wrapped.y * (real)height), height - 1u);
    return ld4(s->texture_pixels[offset + y * width + x]);
}
// fallbackSky / sampleEnvironment: PathTrace.metal:3765-3802
static V3 fallbackSky(V3 d) {
    real sky = K(0.5) * (d.y + K(1.0));
    return mix3(v3(K(0.02), K(0.025), K(0.035)), v3(K(0.25), K(0.32), K(0.45)), sky);
}
static V3 sampleEnvironment(const Ctx& c, V3 direction) {
    count(c, C_ENV_LOOKUPS);
    const dk_scene* s = c.s;
    real intensity = mx((real)s->environment_intensity, K(0.0));
    if (s->environment_texture_index_plus_one == 0u) return fallbackSky(direction) * intensity;
    real sn = std::sin((real)s->environment_rotation_y);
    real cs = std::cos((real)s->environment_rotation_y);
    V3 rotated = normalize(v3(cs * direction.x - sn * direction.z, direction.y, sn * direction.x + cs * direction.z));
    real u = std::atan2(rotated.z, rotated.x) * K(0.15915494309) + K(0.5);
    real v = std::acos(clampf(rotated.y, K(-1.0), K(1.0))) * K(0.31830988618);
    v = clampf(v, K(0.00001), K(0.99999));
    V3 color = sampleTexture(c, s->environment_texture_index_plus_one, v2(u, v), v4(fallbackSky(direction), K(1.0))).xyz() * intensity;
    real maxRadiance = mx((real)s->environment_max_radiance, K(0.0));
    if (maxRadiance > K(0.0)) color = mn(color, v3(maxRadiance));
    return color;
}
// environmentPixelIndexForDirection / environmentPDF: PathTrace.metal:3870-3914
static uint32_t environmentPixelIndexForDirection(const Ctx& c, V3 direction) {
    const dk_scene* s = c.s;
    if (s->environment_texture_index_plus_one == 0u || s->texture_descriptors == nullptr) return 0u;
    const dk_texture_descriptor& d = s->texture_descriptors[s->environment_texture_index_plus_one - 1u];
    uint32_t width = d.metadata.y, height = d.metadata.z;
    if (width == 0u || height == 0u) return 0u;
    real sn = std::sin((real)s->environment_rotation_y);
    real cs = std::cos((real)s->environment_rotation_y);
    V3 rotated = normalize(v3(cs * direction.x - sn * direction.z, direction.y, sn * direction.x + cs * direction.z));
    real u = fractf(std::atan2(rotated.z, rotated.x) * K(0.15915494309) + K(0.5));
    real v = clampf(std::acos(clampf(rotated.y, K(-1.0), K(1.0))) * K(0.31830988618), K(0.0), (real)0.99999994f);
    uint32_t x = std::min((uint32_t)(u * (real)width), width - 1u);
    uint32_t y = std::min((uint32_t)(v * (real)height), height - 1u);
    return y * width + x;
}
static real environmentPDF(const Ctx& c, V3 direction) {
    const dk_scene* s = c.s;
    if (s->environment_samples == nullptr || s->environment_sample_count == 0u) return K(0.0);
    uint32_t index = environmentPixelIndexForDirection(c, direction);
    if (index >= s->environment_sample_count) return K(0.0);
    return mx((real)s->environment_samples[index].pdf_solid_angle, K(0.0));
}
// selectEnvironmentSampleIndex: PathTrace.metal:3916-3935
static uint32_t selectEnvironmentSampleIndex(const Ctx& c, uint32_t count_, real sample) {
    if (count_ <= 1u) return 0u;
    real target = clampf(sample, K(0.0), (real)0.99999994f);
    uint32_t low = 0u, high = count_ - 1u;
    while (low < high) {
        count(c, C_ENV_SEARCH_STEPS);
        uint32_t mid = (low + high) >> 1u;
        if (target <= (real)c.s->environment_samples[mid].cdf) high = mid; else low = mid + 1u;
    }
    return low;
}
// sampleEnvironmentDirection: PathTrace.metal:3937-3987
static V3 sampleEnvironmentDirection(const Ctx& c, V2 pixelSample, real cdfSample, real& pdf) {
    const dk_scene* s = c.s;
    pdf = K(0.0);
    if (s->environment_texture_index_plus_one == 0u || s->environment_sample_count == 0u ||
        s->texture_descriptors == nullptr || s->environment_samples == nullptr)
        return v3(0, 1, 0);
    const dk_texture_descriptor& d = s->texture_descriptors[s->environment_texture_index_plus_one - 1u];
    uint32_t width = d.metadata.y, height = d.metadata.z;
    if (width == 0u || height == 0u) return v3(0, 1, 0);
    count(c, C_ENV_SAMPLES);
    uint32_t index = selectEnvironmentSampleIndex(c, s->environment_sample_count, cdfSample);
    index = std::min(index, s->environment_sample_count - 1u);
    uint32_t x = index % width;
    uint32_t y = index / width;
    real u = ((real)x + pixelSample.x) / (real)width;
    real v = ((real)y + pixelSample.y) / (real)height;
    real phi = (u - K(0.5)) * K(6.28318530718);
    real theta = clampf(v, K(0.00001), K(0.99999)) * K(3.14159265359);
    real sinTheta = std::sin(theta);
    V3 local = normalize(v3(std::cos(phi) * sinTheta, std::cos(theta), std::sin(phi) * sinTheta));
    real sn = std::sin((real)s->environment_rotation_y);
    real cs = std::cos((real)s->environment_rotation_y);
    pdf = mx((real)s->environment_samples[index].pdf_solid_angle, K(0.0));
    return normalize(v3(cs * local.x + sn * local.z, local.y, -sn * local.x + cs * local.z));
}
// applyBaseColorTexture: PathTrace.metal:4005-4019
static Material applyBaseColorTexture(const Ctx& c, Material m, const Hit& hit) {
    uint32_t idx = (uint32_t)m.parameters.z;
    if (idx == 0u) return m;
    V4 texel = sampleTexture(c, idx, hit.uv, v4(1, 1, 1, 1));
    m.baseColor = m.baseColor * texel;
    return m;
}
// applyNormalMap: PathTrace.metal:4021-4054
static Hit applyNormalMap(const Ctx& c, Hit hit, const Material& m, V3 rayDirection) {
    uint32_t idx = (uint32_t)m.parameters.w;
    if (idx == 0u) return hit;
    V3 mapped = sampleTexture(c, idx, hit.uv, v4(K(0.5), K(0.5), K(1.0), K(1.0))).xyz();
    mapped = normalize(mapped * K(2.0) - v3(K(1.0)));
    V3 tangent = hit.tangent - hit.normal * dot(hit.tangent, hit.normal);
    if (length(tangent) <= K(1e-5)) {
        V3 helper = std::fabs(hit.normal.y) < K(0.999) ? v3(0, 1, 0) : v3(1, 0, 0);
        tangent = cross(helper, hit.normal);
    }
    tangent = normalize(tangent);
    V3 bitangent = hit.bitangent - hit.normal * dot(hit.bitangent, hit.normal);
    if (length(bitangent) <= K(1e-5)) bitangent = cross(hit.normal, tangent);
    bitangent = normalize(bitangent);
    hit.normal = normalize(mapped.x * tangent + mapped.y * bitangent + mapped.z * hit.normal);
    if (dot(hit.normal, rayDirection) > K(0.0)) hit.normal = -hit.normal;
    return hit;
}
// makeCameraRay: PathTrace.metal:4056-4091
static Ray makeCameraRay(const dk_camera& cam, uint32_t width, uint32_t height, uint32_t gx, uint32_t gy, real jitterX,
                         real jitterY, real lensX, real lensY) {
    real u = ((real)gx + jitterX) / (real)width;
    real v = K(1.0) - (((real)gy + jitterY) / (real)height);
    Ray ray;
    V3 lowerLeft = ld3(cam.lower_left), horizontal = ld3(cam.horizontal), vertical = ld3(cam.vertical);
    V3 planePoint = lowerLeft + u * horizontal + v * vertical;
    if ((real)cam.origin.w > K(0.5)) {
        ray.origin = planePoint;
        ray.direction = normalize(cross(vertical, horizontal));
    } else {
        ray.origin = ld3(cam.origin);
        ray.direction = normalize(planePoint - ray.origin);
    }
    real apertureRadius = mx((real)cam.lens.x, K(0.0));
    if ((real)cam.origin.w <= K(0.5) && apertureRadius > K(0.0)) {
        V3 forward = normalize(cross(vertical, horizontal));
        real focusDistance = mx((real)cam.lens.y, K(0.0001));
        real focalT = focusDistance / mx(dot(ray.direction, forward), K(0.0001));
        V3 focalPoint = ray.origin + ray.direction * focalT;
        V2 disk = uniformDisk(v2(lensX, lensY)) * apertureRadius;
        V3 right = normalize(horizontal);
        V3 trueUp = normalize(vertical);
        ray.origin += right * disk.x + trueUp * disk.y;
        ray.direction = normalize(focalPoint - ray.origin);
    }
    return ray;
}
// tracePrimaryAOV: PathTrace.metal:4093-4159
static bool tracePrimaryAOV(const Ctx& c, Ray ray, Hit& primaryHit, Material& primaryMaterial) {
    for (uint32_t pass = 0; pass < 32u; ++pass) {
        Hit hit = intersectScene(c, ray, 3);
        if (!hit.hit) return false;
        Material m = materialForHit(c, hit);
        hit = applyNormalMap(c, hit, m, ray.direction);
        m = applyBaseColorTexture(c, m, hit);
        if (m.baseColor.w <= K(0.001)) {
            ray.origin = hit.position + ray.direction * K(0.001);
            continue;
        }
        primaryHit = hit;
        primaryMaterial = m;
        return true;
    }
    return false;
}
// shadowOccluded: PathTrace.metal:4196-4274 (closest-hit walk of <= 8 layers).
static bool shadowOccluded(const Ctx& c, Ray shadowRay, real maxDistance, V3& transmittance) {
    count(c, C_SHADOW_QUERIES);
    real traveled = K(0.0);
    for (uint32_t step = 0; step < 8u; ++step) {
        Hit h = intersectScene(c, shadowRay, 1);
        if (!h.hit || traveled + h.t >= maxDistance) return false;
        Material sm = materialForHit(c, h);
        if (sm.baseColor.w <= K(0.001)) {
            traveled += h.t;
            shadowRay.origin = h.position + shadowRay.direction * K(0.001);
            continue;
        }
        real transmission = materialTransmission(sm);
        if (transmission <= K(0.001)) return true;
        bool insideSolid = !h.frontFacing && !materialThinWalled(sm);
        V3 medium = materialHasVolumeScattering(sm) && insideSolid ? materialVolumeTransmittance(sm, h.t)
                                                                   : materialTransmissionAbsorption(sm, h.t, insideSolid);
        transmittance *= materialTransmissionTint(sm, K(0.35)) * medium * transmission;
        if (maxComponent(transmittance) < K(0.02)) return true;
        traveled += h.t;
        shadowRay.origin = h.position + shadowRay.direction * K(0.001);
    }
    return true;
}
// sampleDirectLighting: PathTrace.metal:4407-4585 (1 emissive-triangle sample
// + 2 environment samples, each with a power-heuristic MIS weight).
static V3 sampleDirectLighting(const Ctx& c, const Hit& hit, const Material& surface, V3 view, uint32_t& state) {
    const dk_scene* s = c.s;
    V3 direct = v3(K(0.0));
    if (s->light_count > 0u && s->lights != nullptr) {
        uint32_t index = selectLightIndex(c, s->light_count, randomFloat(state));
        const dk_light_record& light = s->lights[index];
        real selectionPDF = lightSelectionPDF(c, index);
        uint32_t lti = light.triangle_index;
        if (lti < s->triangle_count && selectionPDF > K(0.0)) {
            const dk_triangle& lt = s->triangles[lti];
            count(c, C_MATERIAL_FETCH);
            Material lm = loadMaterial(s->materials[std::min(light.material_index, s->material_count - 1u)]);
            V3 emission = lm.emission.xyz();
            real area = (real)light.area;
            if (area > K(0.0)) {
                count(c, C_LIGHT_SAMPLES);
                real r0 = randomFloat(state);
                real r1 = randomFloat(state);
                V3 lightPoint = sampleTriangle(lt, v2(r0, r1));
                V3 toLight = lightPoint - hit.position;
                real distanceSquared = dot(toLight, toLight);
                real distanceToLight = std::sqrt(distanceSquared);
                V3 lightDirection = toLight / distanceToLight;
                real cosSurface = mx(K(0.0), dot(hit.normal, lightDirection));
                V3 lightNormal = ld3(light.normal);
                real cosLight = mx(K(0.0), dot(lightNormal, -lightDirection));
                if (cosSurface > K(0.0) && cosLight > K(0.0)) {
                    real lightPDF = selectionPDF * lightSolidAnglePDF(distanceSquared, cosLight, area);
                    real bsdfPDF = materialBSDFPDF(surface, hit.normal, hit.tangent, hit.bitangent, view, lightDirection);
                    real misWeight = powerHeuristic(lightPDF, bsdfPDF);
                    Ray shadowRay;
                    shadowRay.origin = hit.position + hit.normal * K(0.001);
                    shadowRay.direction = lightDirection;
                    V3 shadowT = v3(K(1.0));
                    if (!shadowOccluded(c, shadowRay, distanceToLight - K(0.002), shadowT)) {
                        real geometryTerm = cosSurface * cosLight * area / mx(distanceSquared, K(1e-6));
                        V3 brdf = evaluateMaterialBRDF(surface, hit.normal, hit.tangent, hit.bitangent, view, lightDirection);
                        direct += brdf * emission * geometryTerm * misWeight * shadowT / selectionPDF;
                    }
                }
            }
        }
    }
    const uint32_t envCount = 2u;
    for (uint32_t e = 0u; e < envCount; ++e) {
        real envPDF;
        real a = randomFloat(state);
        real b = randomFloat(state);
        real cdf = randomFloat(state);
        V3 envDir = sampleEnvironmentDirection(c, v2(a, b), cdf, envPDF);
        real envCos = mx(K(0.0), dot(hit.normal, envDir));
        if (envPDF > K(0.0) && envCos > K(0.0)) {
            real bsdfPDF = materialBSDFPDF(surface, hit.normal, hit.tangent, hit.bitangent, view, envDir);
            real misWeight = powerHeuristic(envPDF, bsdfPDF);
            Ray shadowRay;
            shadowRay.origin = hit.position + hit.normal * K(0.001);
            shadowRay.direction = envDir;
            V3 shadowT = v3(K(1.0));
            if (!shadowOccluded(c, shadowRay, K(1.0e20), shadowT)) {
                V3 brdf = evaluateMaterialBRDF(surface, hit.normal, hit.tangent, hit.bitangent, view, envDir);
                V3 envRadiance = sampleEnvironment(c, envDir);
                direct += brdf * envRadiance * envCos * misWeight * shadowT / (envPDF * (real)envCount);
            }
        }
    }
    return direct;
}

struct PixelResult {
    V3 radiance;
    real alpha;
    bool hasAOV;
    Hit aovHit;
    Material aovMaterial;
};

// pathTraceKernel body: PathTrace.metal:5167-5586 for one pixel and sample.
static PixelResult tracePath(const Ctx& c, uint32_t px, uint32_t py, uint32_t sampleIndex) {
    const oracle_params* p = c.p;
    count(c, C_PATHS);
    uint32_t state = p->frame_seed ^ hash_u32(px + py * p->width) ^ hash_u32(sampleIndex + 1u);
    real j0 = randomFloat(state);
    real j1 = randomFloat(state);
    real j2 = randomFloat(state);
    real j3 = randomFloat(state);
    Ray ray = makeCameraRay(p->camera, p->width, p->height, px, py, j0, j1, j2, j3);
    V3 radiance = v3(K(0.0));
    V3 throughput = v3(K(1.0));
    real outputAlpha = K(1.0);
    real previousBSDFPDF = K(0.0);
    Hit primaryHit = emptyHit();
    Material primaryMaterial;
    std::memset(&primaryMaterial, 0, sizeof(primaryMaterial));
    for (uint32_t bounce = 0; bounce < p->max_bounces; ++bounce) {
        count(c, C_BOUNCES);
        Hit hit = intersectScene(c, ray, 0);
        if (!hit.hit) {
            if (p->transparent_background != 0u && !primaryHit.hit) {
                outputAlpha = K(0.0);
            } else if (p->shows_environment_background == 0u && !primaryHit.hit) {
                outputAlpha = K(1.0);
                radiance += mx(v3((real)p->background_color[0], (real)p->background_color[1], (real)p->background_color[2]), v3(K(0.0)));
            } else {
                count(c, C_MISS_ENV);
                real envWeight = K(1.0);
                if (bounce > 0u && previousBSDFPDF > K(0.0)) {
                    real envLightPDF = environmentPDF(c, ray.direction);
                    envWeight = powerHeuristic(previousBSDFPDF, envLightPDF);
                }
                V3 contribution = throughput * sampleEnvironment(c, ray.direction) * envWeight;
                radiance += clampSampleContribution(contribution, c);
            }
            break;
        }
        Material m = materialForHit(c, hit);
        hit = applyNormalMap(c, hit, m, ray.direction);
        m = applyBaseColorTexture(c, m, hit);
        if (m.baseColor.w <= K(0.001)) {
            ray.origin = hit.position + ray.direction * K(0.001);
            continue;
        }
        if (!primaryHit.hit) {
            primaryHit = hit;
            primaryMaterial = m;
        }
        if (continueTransmissionVolumeRandomWalk(hit, m, ray, throughput, previousBSDFPDF, state)) {
            if (terminatePathWithRussianRoulette(bounce, throughput, state)) break;
            continue;
        }
        real subsurface = materialSubsurface(m);
        if (subsurface > K(0.0) && randomFloat(state) < subsurface) {
            if (continueSubsurfaceRandomWalk(c, hit, m, ray, throughput, previousBSDFPDF, state)) {
                if (terminatePathWithRussianRoulette(bounce, throughput, state)) break;
                continue;
            }
        }
        if (continueTransmissiveSurface(hit, m, ray, throughput, previousBSDFPDF, state)) {
            if (terminatePathWithRussianRoulette(bounce, throughput, state)) break;
            continue;
        }
        if (maxComponent(m.emission.xyz()) > K(0.0)) {
            real emissionWeight = K(1.0);
            if (bounce > 0u && previousBSDFPDF > K(0.0)) {
                real lightPDF = lightPDFForHit(c, hit, ray.direction);
                emissionWeight = powerHeuristic(previousBSDFPDF, lightPDF);
            }
            V3 contribution = throughput * m.emission.xyz() * emissionWeight;
            radiance += clampSampleContribution(contribution, c);
            break;
        }
        V3 direct = throughput * sampleDirectLighting(c, hit, m, -ray.direction, state);
        radiance += clampSampleContribution(direct, c);
        real roughness = clampf(m.parameters.x, K(0.02), K(1.0));
        real anisotropy = materialSpecularAnisotropy(m);
        V3 f0 = materialF0(m);
        real clearcoat = materialClearcoat(m);
        real clearcoatRoughness = materialClearcoatRoughness(m);
        real dP, sP, cP;
        materialLobeProbabilities(m, dP, sP, cP);
        real c0 = randomFloat(state);
        real c1 = randomFloat(state);
        V3 localDirection = cosineHemisphere(v2(c0, c1));
        V3 diffuseDirection = orientHemisphere(localDirection, hit.normal);
        V3 nextDirection;
        real lobeSample = randomFloat(state);
        V3 view = -ray.direction;
        if (lobeSample < cP) {
            real a = randomFloat(state);
            real b = randomFloat(state);
            V3 h = sampleGGXVisibleNormal(v2(a, b), hit.normal, hit.tangent, hit.bitangent, view, clearcoatRoughness, K(0.0));
            nextDirection = normalize(reflect(ray.direction, h));
            if (dot(nextDirection, hit.normal) <= K(0.0)) {
                nextDirection = diffuseDirection;
                throughput *= materialDiffuseBounceWeight(m, hit.normal, view, nextDirection) / mx(dP, K(1e-5));
            } else {
                real nDotL = mx(dot(hit.normal, nextDirection), K(1e-5));
                real vDotH = mx(dot(view, h), K(1e-5));
                throughput *= clearcoat * fresnelSchlickThinFilm(vDotH, materialClearcoatF0Color(m), m) *
                              geometrySmithG1GGX(nDotL, clearcoatRoughness) / mx(cP, K(1e-5));
            }
        } else if (lobeSample < cP + sP) {
            real a = randomFloat(state);
            real b = randomFloat(state);
            V3 h = sampleGGXVisibleNormal(v2(a, b), hit.normal, hit.tangent, hit.bitangent, view, roughness, anisotropy);
            nextDirection = normalize(reflect(ray.direction, h));
            if (dot(nextDirection, hit.normal) <= K(0.0)) {
                nextDirection = diffuseDirection;
                throughput *= materialDiffuseBounceWeight(m, hit.normal, view, nextDirection) / mx(dP, K(1e-5));
            } else {
                real vDotH = mx(dot(view, h), K(1e-5));
                V3 fresnel = fresnelSchlickThinFilm(vDotH, f0, m);
                V3 cca = materialClearcoatAttenuationForDirection(m, hit.normal, view, nextDirection);
                throughput *= cca * fresnel *
                              geometrySmithG1GGXAnisotropic(nextDirection, hit.normal, hit.tangent, hit.bitangent, roughness, anisotropy) /
                              mx(sP, K(1e-5));
            }
        } else {
            nextDirection = diffuseDirection;
            throughput *= materialDiffuseBounceWeight(m, hit.normal, view, nextDirection) / mx(dP, K(1e-5));
        }
        previousBSDFPDF = materialBSDFPDF(m, hit.normal, hit.tangent, hit.bitangent, view, nextDirection);
        ray.origin = hit.position + hit.normal * K(0.001);
        ray.direction = nextDirection;
        if (terminatePathWithRussianRoulette(bounce, throughput, state)) break;
    }
    PixelResult r;
    r.radiance = radiance;
    r.alpha = outputAlpha;
    r.hasAOV = primaryHit.hit;
    r.aovHit = primaryHit;
    r.aovMaterial = primaryMaterial;
    if (p->denoiser_enabled != 0u) {
        Ray aovRay = makeCameraRay(p->camera, p->width, p->height, px, py, K(0.5), K(0.5), K(0.0), K(0.0));
        r.hasAOV = tracePrimaryAOV(c, aovRay, r.aovHit, r.aovMaterial);
    }
    return r;
}

// AOV block: PathTrace.metal:5559-5585.  Stores into six RGBA planes in the
// order depth, normal, albedo, materialID, objectID, motionVector.
static void writeAOVs(const Ctx& c, const PixelResult& r, uint32_t px, uint32_t py, float* aov, size_t plane) {
    const oracle_params* p = c.p;
    size_t o = ((size_t)py * p->width + px) * 4;
    float* depth = aov + 0 * plane + o;
    float* normal = aov + 1 * plane + o;
    float* albedo = aov + 2 * plane + o;
    float* matID = aov + 3 * plane + o;
    float* objID = aov + 4 * plane + o;
    float* motion = aov + 5 * plane + o;
    auto put = [](float* d, real a, real b, real cc, real w) { d[0] = (float)a; d[1] = (float)b; d[2] = (float)cc; d[3] = (float)w; };
    if (r.hasAOV) {
        const Hit& h = r.aovHit;
        V3 enc = h.normal * K(0.5) + v3(K(0.5));
        put(depth, h.t, h.t, h.t, K(1.0));
        put(normal, enc.x, enc.y, enc.z, K(1.0));
        put(albedo, r.aovMaterial.baseColor.x, r.aovMaterial.baseColor.y, r.aovMaterial.baseColor.z, r.aovMaterial.baseColor.w);
        real mid = (real)(float)(h.materialID + 1u);
        real oid = (real)(float)(h.objectID + 1u);
        put(matID, mid, mid, mid, K(1.0));
        put(objID, oid, oid, oid, K(1.0));
        V2 cur, prev;
        if (projectToScreen(p->camera, h.position, p->width, p->height, cur) &&
            projectToScreen(p->previous_camera, h.position, p->width, p->height, prev)) {
            V2 motion2 = prev - cur;
            put(motion, motion2.x, motion2.y, K(0.0), K(1.0));
        } else {
            put(motion, 0, 0, 0, 0);
        }
    } else {
        put(depth, 0, 0, 0, 0);
        put(normal, K(0.5), K(0.5), K(0.5), K(0.0));
        put(albedo, 0, 0, 0, 0);
        put(matID, 0, 0, 0, 0);
        put(objID, 0, 0, 0, 0);
        put(motion, 0, 0, 0, 0);
    }
}

}  // namespace

// =========================================================== C exports ====
extern "C" {

#if defined(ORACLE_FP64)
#define ORACLE_EXPORT(name) oracle64_##name
#else
#define ORACLE_EXPORT(name) oracle32_##name
#endif

uint32_t ORACLE_EXPORT(hash)(uint32_t v) { return hash_u32(v); }

// Draws `n` values of randomFloat from `state` (for RNG known-answer tests).
void ORACLE_EXPORT(random_sequence)(uint32_t state, uint32_t n, double* out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = (double)randomFloat(state);
}

// Renders samples [sample_begin, sample_begin + sample_count) of the pixels of
// the tile in `p` (or of `pixel_list` when it is non-null), updating the
// running mean `accum` (RGBA per pixel, W*H*4 doubles; PathTrace.metal:
// 5520-5524, rounded to float per sample in the FP32 build as the RGBA32F
// texture does) and the last-sample AOV planes (6 * W*H*4 floats, may be null).
// `counters` (C_COUNT entries) accumulates work counts; `threads` <= 0 uses all
// hardware threads.  Returns 0 on success, 1 for a null argument, 2 for an
// empty image, 3 for a scene without materials and 4 when a listed pixel lies
// outside the image (nothing is written then).
int ORACLE_EXPORT(render)(const dk_scene* scene, const oracle_params* params, uint32_t sample_begin,
                          uint32_t sample_count, const uint32_t* pixel_list, uint32_t pixel_list_count, int threads,
                          double* accum, float* aov, uint64_t* counters) {
    if (!scene || !params || !accum) return 1;
    if (scene->material_count == 0) return 3;
    if (params->width == 0 || params->height == 0) return 2;
    std::vector<uint32_t> pixels;
    if (pixel_list) {
        // Every listed pixel must lie in the W*H image the buffers hold.
        const uint64_t npix = (uint64_t)params->width * params->height;
        for (uint32_t i = 0; i < pixel_list_count; ++i)
            if (pixel_list[i] >= npix) return 4;
        pixels.assign(pixel_list, pixel_list + pixel_list_count);
    } else {
        for (uint32_t y = params->tile_y; y < params->tile_y + params->tile_h && y < params->height; ++y)
            for (uint32_t x = params->tile_x; x < params->tile_x + params->tile_w && x < params->width; ++x)
                pixels.push_back(y * params->width + x);
    }
    int nthreads = threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<size_t> next(0);
    std::vector<Counters> per(nthreads);
    const size_t plane = (size_t)params->width * params->height * 4;
    auto worker = [&](int tid) {
        Counters& cnt = per[tid];
        std::memset(&cnt, 0, sizeof(cnt));
        Ctx ctx{scene, params, &cnt};
        const size_t chunk = 64;
        for (;;) {
            size_t begin = next.fetch_add(chunk);
            if (begin >= pixels.size()) break;
            size_t end = std::min(pixels.size(), begin + chunk);
            for (size_t i = begin; i < end; ++i) {
                uint32_t pix = pixels[i];
                uint32_t px = pix % params->width, py = pix / params->width;
                double* a = accum + (size_t)pix * 4;
                PixelResult last{};
                for (uint32_t s = sample_begin; s < sample_begin + sample_count; ++s) {
                    PixelResult r = tracePath(ctx, px, py, s);
                    real w = K(1.0) / ((real)s + K(1.0));
                    real prev[4] = {(real)a[0], (real)a[1], (real)a[2], (real)a[3]};
                    real cur[4] = {r.radiance.x, r.radiance.y, r.radiance.z, r.alpha};
                    for (int k = 0; k < 4; ++k) {
                        real v = mixf(prev[k], cur[k], w);
#if !defined(ORACLE_FP64)
                        v = (float)v;
#endif
                        a[k] = (double)v;
                    }
                    last = r;
                }
                if (aov && sample_count > 0) writeAOVs(ctx, last, px, py, aov, plane);
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nthreads; ++t) pool.emplace_back(worker, t);
    worker(0);
    for (auto& t : pool) t.join();
    if (counters)
        for (auto& cnt : per)
            for (int k = 0; k < C_COUNT; ++k) counters[k] += cnt.c[k];
    return 0;
}

// Closest hit of one ray (intersectScene, PathTrace.metal:3294-3421).  out_hit
// receives {hit, t, px, py, pz, nx, ny, nz, u, v, materialID, objectID,
// primitiveID, frontFacing}.
int ORACLE_EXPORT(intersect)(const dk_scene* scene, const float* origin, const float* direction, double* out_hit) {
    Counters cnt;
    std::memset(&cnt, 0, sizeof(cnt));
    oracle_params p;
    std::memset(&p, 0, sizeof(p));
    Ctx ctx{scene, &p, &cnt};
    Ray ray;
    ray.origin = v3(origin[0], origin[1], origin[2]);
    ray.direction = v3(direction[0], direction[1], direction[2]);
    Hit h = intersectScene(ctx, ray, 0);
    double v[14] = {h.hit ? 1.0 : 0.0, (double)h.t, (double)h.position.x, (double)h.position.y, (double)h.position.z,
                    (double)h.normal.x, (double)h.normal.y, (double)h.normal.z, (double)h.uv.x, (double)h.uv.y,
                    (double)h.materialID, (double)h.objectID, (double)h.primitiveID, h.frontFacing ? 1.0 : 0.0};
    std::memcpy(out_hit, v, sizeof(v));
    return 0;
}

uint32_t ORACLE_EXPORT(counter_count)(void) { return C_COUNT; }

}  // extern "C"
