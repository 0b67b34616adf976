// Layered BSDF, lights, environment and random walks of the sm_103a path
// tracer, restating the reference shader function by function
// (Sources/DenrimRendererKit/Resources/Shaders/PathTrace.metal; line ranges
// beside each function).  Every randomFloat draw happens in the reference's
// left-to-right textual order, so a path consumes the same RNG stream.
#pragma once
#include "dk_device.cuh"

namespace dk {

struct Material {
    float4 baseColor, emission, parameters, parameters2, specularColor, sheenColor, transmissionColor,
        parameters3, clearcoatColor, clearcoatAttenuation, transmissionAbsorption, thinFilm, subsurfaceColor,
        subsurfaceRadius, subsurfaceParameters, volumeScattering, volumeParameters;
};

__device__ __forceinline__ Material loadMaterial(const dk_material* mats, uint32_t i) {
    const float4* p = reinterpret_cast<const float4*>(mats + i);
    Material m;
    m.baseColor = __ldg(p + 0);
    m.emission = __ldg(p + 1);
    m.parameters = __ldg(p + 2);
    m.parameters2 = __ldg(p + 3);
    m.specularColor = __ldg(p + 4);
    m.sheenColor = __ldg(p + 5);
    m.transmissionColor = __ldg(p + 6);
    m.parameters3 = __ldg(p + 7);
    m.clearcoatColor = __ldg(p + 8);
    m.clearcoatAttenuation = __ldg(p + 9);
    m.transmissionAbsorption = __ldg(p + 10);
    m.thinFilm = __ldg(p + 11);
    m.subsurfaceColor = __ldg(p + 12);
    m.subsurfaceRadius = __ldg(p + 13);
    m.subsurfaceParameters = __ldg(p + 14);
    m.volumeScattering = __ldg(p + 15);
    m.volumeParameters = __ldg(p + 16);
    return m;
}

// ------------------------------------------------- sampling helpers -------
__device__ __forceinline__ float3 cosineHemisphere(float ux, float uy) {  // :270-275
    float r = sqrtf(ux);
    float phi = 6.28318530718f * uy;
    float s, c;
    sincosf(phi, &s, &c);
    return f3(r * c, r * s, sqrtf(fmaxf(0.0f, 1.0f - ux)));
}
__device__ __forceinline__ float2 uniformDisk(float ux, float uy) {  // :277-281
    float r = sqrtf(ux);
    float s, c;
    sincosf(6.28318530718f * uy, &s, &c);
    return make_float2(r * c, r * s);
}
__device__ __forceinline__ float3 uniformSphere(float ux, float uy) {  // :283-288
    float z = 1.0f - 2.0f * ux;
    float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float s, c;
    sincosf(6.28318530718f * uy, &s, &c);
    return f3(r * c, r * s, z);
}
__device__ __forceinline__ float3 orientHemisphere(float3 l, float3 n) {  // :290-295
    float3 helper = fabsf(n.y) < 0.999f ? f3(0, 1, 0) : f3(1, 0, 0);
    float3 t = normalize(cross(helper, n));
    float3 b = cross(n, t);
    return normalize(l.x * t + l.y * b + l.z * n);
}
__device__ __forceinline__ float3 sampleHenyeyGreenstein(float ux, float uy, float3 dir, float anisotropy) {  // :304-318
    float g = clampf(anisotropy, -0.95f, 0.95f);
    if (fabsf(g) < 1e-4f) return uniformSphere(ux, uy);
    float omg2 = 1.0f - g * g;
    float q = omg2 / fmaxf(1.0f - g + 2.0f * g * ux, 1e-5f);
    float cosT = clampf((1.0f + g * g - q * q) / (2.0f * g), -1.0f, 1.0f);
    float sinT = sqrtf(fmaxf(0.0f, 1.0f - cosT * cosT));
    float s, c;
    sincosf(6.28318530718f * uy, &s, &c);
    return orientHemisphere(f3(c * sinT, s * sinT, cosT), dir);  // orientAroundDirection == orientHemisphere
}
__device__ __forceinline__ float3 clampSampleContribution(float3 c, float clampParam) {  // :324-340
    if (!allFinite(c)) return f3(0.0f);
    float cv = fmaxf(clampParam, 0.0f);
    if (cv <= 0.0f) return c;
    float peak = maxComponent(c);
    if (peak <= cv) return c;
    return c * (cv / fmaxf(peak, 1e-5f));
}
__device__ __forceinline__ float luminance(float3 v) { return dot(v, f3(0.2126f, 0.7152f, 0.0722f)); }

// ---------------------------------------------------- material model ------
__device__ __forceinline__ float3 fresnelSchlick(float cosT, float3 f0) {  // :346-349
    float x = clampf(1.0f - cosT, 0.0f, 1.0f);
    float x2 = x * x;
    float factor = x2 * x2 * x;  // pow(x, 5)
    return f0 + (f3(1.0f) - f0) * factor;
}
__device__ float3 thinFilmTint(const Material& m, float cosT) {  // :351-370
    float strength = clampf(m.thinFilm.x, 0.0f, 1.0f);
    float thickness = fmaxf(m.thinFilm.y, 0.0f);
    if (strength <= 0.0f || thickness <= 0.0f) return f3(1.0f);
    float filmIOR = fmaxf(m.thinFilm.z, 1.0001f);
    float angle = powf(clampf(1.0f - cosT, 0.0f, 1.0f), 0.65f);
    float opticalPath = 2.0f * filmIOR * thickness * (0.62f + 0.42f * angle);
    float3 phase = 6.28318530718f * opticalPath / f3(650.0f, 510.0f, 475.0f);
    float3 interference = f3(0.62f + 0.38f * cosf(phase.x), 0.62f + 0.38f * cosf(phase.y), 0.62f + 0.38f * cosf(phase.z));
    float nl = fmaxf(luminance(interference), 0.35f);
    float3 tint = clamp3(interference / nl, f3(0.35f), f3(1.8f));
    return mix3(f3(1.0f), tint, strength);
}
__device__ __forceinline__ float3 fresnelSchlickThinFilm(float cosT, float3 f0, const Material& m) {
    return fresnelSchlick(cosT, f0) * thinFilmTint(m, cosT);
}
__device__ float dielectricFresnel(float cosI, float etaI, float etaT) {  // :378-393
    cosI = clampf(cosI, 0.0f, 1.0f);
    float eta = etaI / etaT;
    float s2 = eta * eta * fmaxf(0.0f, 1.0f - cosI * cosI);
    if (s2 >= 1.0f) return 1.0f;
    float cosT = sqrtf(fmaxf(0.0f, 1.0f - s2));
    float par = ((etaT * cosI) - (etaI * cosT)) / fmaxf((etaT * cosI) + (etaI * cosT), 1e-5f);
    float per = ((etaI * cosI) - (etaT * cosT)) / fmaxf((etaI * cosI) + (etaT * cosT), 1e-5f);
    return clampf(0.5f * (par * par + per * per), 0.0f, 1.0f);
}
__device__ __forceinline__ float dielectricF0(float ior_, float w) {  // :395-399
    float ior = fmaxf(ior_, 1.0f);
    float f0 = (ior - 1.0f) / (ior + 1.0f);
    return f0 * f0 * clampf(w, 0.0f, 1.0f);
}
__device__ __forceinline__ float3 materialF0(const Material& m) {  // :401-406
    float metallic = clampf(m.parameters.y, 0.0f, 1.0f);
    float d = dielectricF0(m.parameters2.y, m.parameters2.x);
    return mix3(d * clamp3(xyz(m.specularColor), f3(0.0f), f3(1.0f)), xyz(m.baseColor), metallic);
}
__device__ __forceinline__ float materialClearcoat(const Material& m) { return clampf(m.parameters2.z, 0.0f, 1.0f); }
__device__ __forceinline__ float materialClearcoatRoughness(const Material& m) { return clampf(m.parameters2.w, 0.02f, 1.0f); }
__device__ __forceinline__ float3 materialClearcoatF0Color(const Material& m) {
    return dielectricF0(m.specularColor.w, 1.0f) * clamp3(xyz(m.clearcoatColor), f3(0.0f), f3(1.0f));
}
__device__ float3 materialClearcoatDepthAttenuation(const Material& m, float3 n, float3 v, float3 l) {  // :442-456
    float thickness = fmaxf(m.clearcoatAttenuation.w, 0.0f) * materialClearcoat(m);
    if (thickness <= 1e-5f) return f3(1.0f);
    float nDotV = fmaxf(dot(n, v), 0.05f);
    float nDotL = fmaxf(dot(n, l), 0.05f);
    float pathLength = thickness * 0.5f * (1.0f / nDotV + 1.0f / nDotL);
    return exp3(log3(clamp3(xyz(m.clearcoatAttenuation), f3(0.0001f), f3(1.0f))) * pathLength);
}
__device__ __forceinline__ float materialSpecularAnisotropy(const Material& m) { return clampf(m.parameters3.w, -0.95f, 0.95f); }
__device__ __forceinline__ float materialTransmission(const Material& m) { return clampf(m.emission.w, 0.0f, 1.0f); }
__device__ __forceinline__ bool materialThinWalled(const Material& m) { return m.transmissionColor.w > 0.5f; }
__device__ __forceinline__ float materialSheen(const Material& m) { return clampf(m.sheenColor.w, 0.0f, 1.0f); }
__device__ __forceinline__ float3 materialSheenColor(const Material& m) { return clamp3(xyz(m.sheenColor), f3(0.0f), f3(1.0f)); }
__device__ __forceinline__ float materialSubsurface(const Material& m) {
    float metallic = clampf(m.parameters.y, 0.0f, 1.0f);
    return clampf(m.subsurfaceColor.w, 0.0f, 1.0f) * (1.0f - metallic) * (1.0f - materialTransmission(m));
}
__device__ __forceinline__ float3 materialTransmissionTint(const Material& m, float strength) {
    return mix3(f3(1.0f), clamp3(xyz(m.transmissionColor), f3(0.0f), f3(1.0f)), strength);
}
__device__ __forceinline__ float3 materialTransmissionAbsorptionCoefficient(const Material& m) {  // :496-504
    float rd = m.transmissionAbsorption.w;
    if (rd <= 1e-5f) return f3(0.0f);
    return (-log3(clamp3(xyz(m.transmissionAbsorption), f3(0.0001f), f3(1.0f)))) / rd;
}
__device__ __forceinline__ float3 materialTransmissionAbsorption(const Material& m, float d, bool applies) {
    if (!applies || d <= 0.0f) return f3(1.0f);
    return exp3((-materialTransmissionAbsorptionCoefficient(m)) * d);
}
__device__ __forceinline__ float materialVolumeScattering(const Material& m) { return clampf(m.volumeScattering.w, 0.0f, 1.0f); }
__device__ __forceinline__ bool materialHasVolumeScattering(const Material& m) {
    return materialTransmission(m) > 0.0f && !materialThinWalled(m) && materialVolumeScattering(m) > 0.0f;
}
__device__ __forceinline__ float3 materialVolumeSigmaS(const Material& m) {  // :1137-1141
    return clamp3(xyz(m.volumeScattering), f3(0.0f), f3(1.0f)) * materialVolumeScattering(m) / fmaxf(m.volumeParameters.x, 1e-4f);
}
__device__ __forceinline__ float3 materialVolumeSigmaT(const Material& m) {
    return materialTransmissionAbsorptionCoefficient(m) + materialVolumeSigmaS(m);
}

struct TangentFrame { float3 tangent, bitangent; };
__device__ TangentFrame makeTangentFrame(float3 n, float3 rt, float3 rb) {  // :1157-1176
    TangentFrame f;
    float3 t = rt - n * dot(rt, n);
    if (dot(t, t) <= 1e-8f) {
        float3 helper = fabsf(n.y) < 0.999f ? f3(0, 1, 0) : f3(1, 0, 0);
        t = cross(helper, n);
    }
    f.tangent = normalize(t);
    float3 b = rb - n * dot(rb, n) - f.tangent * dot(rb, f.tangent);
    if (dot(b, b) <= 1e-8f) b = cross(n, f.tangent);
    f.bitangent = normalize(b);
    return f;
}
__device__ __forceinline__ float2 anisotropicGGXAlpha(float roughness, float anisotropy) {  // :1178-1187
    float alpha = fmaxf(roughness * roughness, 0.001f);
    float amount = clampf(anisotropy, -0.95f, 0.95f);
    float aspect = sqrtf(fmaxf(0.1f, 1.0f - 0.9f * fabsf(amount)));
    float aL = alpha / aspect, aS = alpha * aspect;
    return amount >= 0.0f ? make_float2(aL, aS) : make_float2(aS, aL);
}
__device__ __forceinline__ float distributionGGX(float nDotH, float roughness) {  // :1189-1194
    float a = roughness * roughness;
    float a2 = a * a;
    float den = nDotH * nDotH * (a2 - 1.0f) + 1.0f;
    return a2 / fmaxf(3.14159265359f * den * den, 1e-5f);
}
__device__ __forceinline__ float geometrySmithG1GGX(float nDotV, float roughness) {  // :1196-1201
    float a = roughness * roughness;
    float a2 = a * a;
    float den = nDotV + sqrtf(fmaxf(a2 + (1.0f - a2) * nDotV * nDotV, 0.0f));
    return (2.0f * nDotV) / fmaxf(den, 1e-5f);
}
__device__ float geometrySmithG1GGXAnisotropic(float3 d, float3 n, float3 t, float3 b, float r, float an) {  // :1229-1250
    float nDotD = fmaxf(dot(n, d), 0.0f);
    if (nDotD <= 0.0f) return 0.0f;
    float2 a = anisotropicGGXAlpha(r, an);
    float tD = dot(t, d), bD = dot(b, d);
    float root = sqrtf(fmaxf(a.x * a.x * tD * tD + a.y * a.y * bD * bD + nDotD * nDotD, 0.0f));
    return (2.0f * nDotD) / fmaxf(nDotD + root, 1e-5f);
}
__device__ float3 evaluateMaterialSheenBRDF(const Material& m, float3 n, float3 v, float3 l) {  // :1266-1297
    float sheen = materialSheen(m);
    if (sheen <= 0.0f) return f3(0.0f);
    float metallic = clampf(m.parameters.y, 0.0f, 1.0f);
    float3 hd = v + l;
    if (dot(hd, hd) <= 1e-8f) return f3(0.0f);
    float3 h = normalize(hd);
    float nDotL = fmaxf(dot(n, l), 0.0f), nDotV = fmaxf(dot(n, v), 0.0f), nDotH = fmaxf(dot(n, h), 0.0f);
    if (nDotL <= 0.0f || nDotV <= 0.0f) return f3(0.0f);
    float sinThetaH = sqrtf(fmaxf(0.0f, 1.0f - nDotH * nDotH));
    float invAlpha = mixf(20.0f, 0.5f, clampf(m.parameters3.x, 0.02f, 1.0f));
    float distribution = (2.0f + invAlpha) * powf(sinThetaH, invAlpha) * 0.15915494309f;
    float visibility = 1.0f / fmaxf(4.0f * (nDotL + nDotV - nDotL * nDotV), 1e-5f);
    return sheen * (1.0f - metallic) * materialSheenColor(m) * distribution * visibility;
}
__device__ float3 materialClearcoatAttenuationForDirection(const Material& m, float3 n, float3 v, float3 l) {  // :1299-1321
    float clearcoat = materialClearcoat(m);
    if (clearcoat <= 0.0f) return f3(1.0f);
    float3 hd = v + l;
    if (dot(hd, hd) <= 1e-8f) return f3(1.0f);
    float3 h = normalize(hd);
    float vDotH = fmaxf(dot(v, h), 0.0f);
    float3 ccF = fresnelSchlickThinFilm(vDotH, materialClearcoatF0Color(m), m);
    float3 att = mx(f3(0.0f), f3(1.0f) - ccF * clearcoat);
    return att * materialClearcoatDepthAttenuation(m, n, v, l);
}
__device__ __forceinline__ float powerHeuristic(float a, float b) {  // :1386-1390
    float a2 = a * a, b2 = b * b;
    return a2 / fmaxf(a2 + b2, 1e-8f);
}
__device__ void materialLobeProbabilities(const Material& m, float& dP, float& sP, float& cP) {  // :1392-1422
    float metallic = clampf(m.parameters.y, 0.0f, 1.0f);
    float3 f0 = materialF0(m);
    float clearcoat = materialClearcoat(m);
    float sheenW = materialSheen(m) * luminance(materialSheenColor(m)) * (1.0f - metallic);
    float diffuseW = luminance(xyz(m.baseColor) * (1.0f - metallic)) + sheenW;
    float specularW = luminance(f0);
    float ccW = clearcoat * luminance(materialClearcoatF0Color(m));
    float total = fmaxf(diffuseW + specularW + ccW, 1e-5f);
    cP = ccW > 1e-5f ? clampf(ccW / total, 0.02f, 0.35f) : 0.0f;
    float remaining = fmaxf(0.0f, 1.0f - cP);
    if (specularW <= 1e-5f) sP = 0.0f;
    else if (diffuseW <= 1e-5f) sP = remaining;
    else sP = clampf(specularW / total, 0.08f, remaining);
    dP = fmaxf(0.0f, 1.0f - sP - cP);
}
__device__ __forceinline__ bool terminatePathWithRussianRoulette(uint32_t bounce, float3& tp, uint32_t& state) {  // :1520-1540
    float w = maxComponent(tp);
    if (w <= 0.0f) return true;
    if (bounce < 2u) return false;
    float survival = clampf(w, 0.05f, 0.95f);
    if (randomFloat(state) > survival) return true;
    tp /= survival;
    return false;
}

// ------------------------------------------------ per-shading-point cache --
// The reference re-derives the tangent frame, GGX alphas, lobe probabilities
// and the view-side Smith terms inside every BRDF / PDF evaluation (three NEE
// directions, the sampled direction and its PDF).  They depend only on the
// shading point, so they are computed once here; each evaluation below then
// performs the remaining operations of evaluateMaterialBRDF (:1323-1384),
// materialBSDFPDF (:1445-1490) and materialDiffuseBounceWeight (:1492-1518)
// in the reference's order.
struct ShadePoint {
    float3 n, t, b, v;      // normal, raw tangent/bitangent, view direction
    TangentFrame fr;        // makeTangentFrame(n, t, b)
    float nDotV;            // max(dot(n, v), 0)
    float roughness, metallic, clearcoat, ccR, anisotropy;
    float3 baseColor, f0, ccF0;
    float2 specAlpha, ccAlpha;
    float g1vSpecAniso, g1vCCAniso, g1vCCIso;
    float dP, sP, cP;
};

__device__ __forceinline__ float distributionGGXAnisotropicA(float3 h, float3 n, float3 t, float3 b, float2 a) {
    float nDotH = fmaxf(dot(n, h), 0.0f);
    if (nDotH <= 0.0f) return 0.0f;
    float tDotH = dot(t, h), bDotH = dot(b, h);
    float den = (tDotH * tDotH) / fmaxf(a.x * a.x, 1e-6f) + (bDotH * bDotH) / fmaxf(a.y * a.y, 1e-6f) + nDotH * nDotH;
    return 1.0f / fmaxf(3.14159265359f * a.x * a.y * den * den, 1e-6f);
}
__device__ __forceinline__ float g1AnisoA(float3 d, float3 n, float3 t, float3 b, float2 a) {
    float nDotD = fmaxf(dot(n, d), 0.0f);
    if (nDotD <= 0.0f) return 0.0f;
    float tD = dot(t, d), bD = dot(b, d);
    float root = sqrtf(fmaxf(a.x * a.x * tD * tD + a.y * a.y * bD * bD + nDotD * nDotD, 0.0f));
    return (2.0f * nDotD) / fmaxf(nDotD + root, 1e-5f);
}

__device__ void makeShadePoint(ShadePoint& sp, const Material& m, float3 n, float3 t, float3 b, float3 v) {
    sp.n = n;
    sp.t = t;
    sp.b = b;
    sp.v = v;
    sp.fr = makeTangentFrame(n, t, b);
    sp.nDotV = fmaxf(dot(n, v), 0.0f);
    sp.roughness = clampf(m.parameters.x, 0.02f, 1.0f);
    sp.metallic = clampf(m.parameters.y, 0.0f, 1.0f);
    sp.clearcoat = materialClearcoat(m);
    sp.ccR = materialClearcoatRoughness(m);
    sp.anisotropy = materialSpecularAnisotropy(m);
    sp.baseColor = xyz(m.baseColor);
    sp.f0 = materialF0(m);
    sp.ccF0 = materialClearcoatF0Color(m);
    sp.specAlpha = anisotropicGGXAlpha(sp.roughness, sp.anisotropy);
    sp.ccAlpha = anisotropicGGXAlpha(sp.ccR, 0.0f);
    sp.g1vSpecAniso = g1AnisoA(v, n, sp.fr.tangent, sp.fr.bitangent, sp.specAlpha);
    sp.g1vCCAniso = g1AnisoA(v, n, sp.fr.tangent, sp.fr.bitangent, sp.ccAlpha);
    sp.g1vCCIso = geometrySmithG1GGX(sp.nDotV, sp.ccR);
    materialLobeProbabilities(m, sp.dP, sp.sP, sp.cP);
}

// materialClearcoatAttenuationForDirection with the clearcoat Fresnel at the
// already-known half vector.
__device__ __forceinline__ float3 clearcoatAttenuationAt(const Material& m, const ShadePoint& sp, float3 l,
                                                         float3 ccFresnel, bool halfOk) {
    if (sp.clearcoat <= 0.0f || !halfOk) return f3(1.0f);
    float3 att = mx(f3(0.0f), f3(1.0f) - ccFresnel * sp.clearcoat);
    return att * materialClearcoatDepthAttenuation(m, sp.n, sp.v, l);
}

__device__ __forceinline__ float3 evalBRDF(const Material& m, const ShadePoint& sp, float3 l) {  // :1323-1384
    const float inversePi = 0.31830988618f;
    float3 hd = sp.v + l;
    float3 h = normalize(hd);
    float nDotL = fmaxf(dot(sp.n, l), 0.0f);
    float nDotH = fmaxf(dot(sp.n, h), 0.0f), vDotH = fmaxf(dot(sp.v, h), 0.0f);
    if (nDotL <= 0.0f || sp.nDotV <= 0.0f) return f3(0.0f);
    float3 tint = thinFilmTint(m, vDotH);
    float3 fresnel = fresnelSchlick(vDotH, sp.f0) * tint;
    float D = distributionGGXAnisotropicA(h, sp.n, sp.fr.tangent, sp.fr.bitangent, sp.specAlpha);
    float G = sp.g1vSpecAniso * g1AnisoA(l, sp.n, sp.fr.tangent, sp.fr.bitangent, sp.specAlpha);
    float3 specular = D * G * fresnel / fmaxf(4.0f * sp.nDotV * nDotL, 1e-5f);
    // The clearcoat lobe is finite, so with clearcoat 0 its weighted term is
    // exactly 0 and is skipped (a warp of one material takes one branch).
    float3 diffuseBase = (f3(1.0f) - fresnel) * (1.0f - sp.metallic) * sp.baseColor * inversePi;
    float3 sheen = evaluateMaterialSheenBRDF(m, sp.n, sp.v, l);
    if (sp.clearcoat <= 0.0f) return diffuseBase + (specular + sheen);
    float3 ccFresnel = fresnelSchlick(vDotH, sp.ccF0) * tint;
    float ccD = distributionGGX(nDotH, sp.ccR);
    float ccG = sp.g1vCCIso * geometrySmithG1GGX(nDotL, sp.ccR);
    float3 ccSpecular = ccD * ccG * ccFresnel / fmaxf(4.0f * sp.nDotV * nDotL, 1e-5f);
    float3 ccAtt = clearcoatAttenuationAt(m, sp, l, ccFresnel, dot(hd, hd) > 1e-8f);
    float3 diffuse = ccAtt * (f3(1.0f) - fresnel) * (1.0f - sp.metallic) * sp.baseColor * inversePi;
    return diffuse + ccAtt * (specular + sheen) + ccSpecular * sp.clearcoat;
}

__device__ __forceinline__ float ggxPDFAt(const ShadePoint& sp, float3 h, float nDotH, float vDotH, float2 a,
                                          float g1v) {  // ggxReflectionPDF (:1424-1443)
    if (nDotH <= 0.0f || sp.nDotV <= 0.0f || vDotH <= 0.0f) return 0.0f;
    return distributionGGXAnisotropicA(h, sp.n, sp.fr.tangent, sp.fr.bitangent, a) * g1v / fmaxf(4.0f * sp.nDotV, 1e-5f);
}

__device__ __forceinline__ float bsdfPDF(const ShadePoint& sp, float3 l) {  // :1445-1490
    float nDotL = fmaxf(dot(sp.n, l), 0.0f);
    if (nDotL <= 0.0f || sp.nDotV <= 0.0f) return 0.0f;
    float3 h = normalize(sp.v + l);
    float nDotH = fmaxf(dot(sp.n, h), 0.0f), vDotH = fmaxf(dot(sp.v, h), 0.0f);
    float specPDF = ggxPDFAt(sp, h, nDotH, vDotH, sp.specAlpha, sp.g1vSpecAniso);
    float ccPDF = sp.cP > 0.0f ? ggxPDFAt(sp, h, nDotH, vDotH, sp.ccAlpha, sp.g1vCCAniso) : 0.0f;
    return sp.dP * (nDotL * 0.31830988618f) + sp.sP * specPDF + sp.cP * ccPDF;
}

__device__ __forceinline__ float3 diffuseBounceWeight(const Material& m, const ShadePoint& sp, float3 l) {  // :1492-1518
    float3 hd = sp.v + l;
    if (dot(hd, hd) <= 1e-8f) return f3(0.0f);
    float3 h = normalize(hd);
    float vDotH = fmaxf(dot(sp.v, h), 0.0f);
    float3 tint = thinFilmTint(m, vDotH);
    float3 fresnel = fresnelSchlick(vDotH, sp.f0) * tint;
    float3 ccAtt = clearcoatAttenuationAt(m, sp, l, fresnelSchlick(vDotH, sp.ccF0) * tint, true);
    float3 diffuse = (f3(1.0f) - fresnel) * (1.0f - sp.metallic) * sp.baseColor;
    float3 sheen = evaluateMaterialSheenBRDF(m, sp.n, sp.v, l) * 3.14159265359f;
    return ccAtt * (diffuse + sheen);
}

// sampleGGXVisibleNormal (:1620-1660) with the shading point's frame.
__device__ __forceinline__ float3 sampleVNDF(const ShadePoint& sp, float ux, float uy, float2 a) {
    float3 lv = normalize(f3(dot(sp.v, sp.fr.tangent), dot(sp.v, sp.fr.bitangent), fmaxf(dot(sp.v, sp.n), 1e-5f)));
    float3 sv = normalize(f3(a.x * lv.x, a.y * lv.y, lv.z));
    float lensq = sv.x * sv.x + sv.y * sv.y;
    float3 t1 = lensq > 1e-7f ? f3(-sv.y, sv.x, 0.0f) * (1.0f / sqrtf(lensq)) : f3(1, 0, 0);
    float3 t2 = cross(sv, t1);
    float radius = sqrtf(ux);
    float s, c;
    sincosf(6.28318530718f * uy, &s, &c);
    float p1 = radius * c;
    float p2 = radius * s;
    float blend = 0.5f * (1.0f + sv.z);
    p2 = mixf(sqrtf(fmaxf(0.0f, 1.0f - p1 * p1)), p2, blend);
    float3 vn = p1 * t1 + p2 * t2 + sqrtf(fmaxf(0.0f, 1.0f - p1 * p1 - p2 * p2)) * sv;
    float3 lh = normalize(f3(a.x * vn.x, a.y * vn.y, fmaxf(vn.z, 0.0f)));
    return normalize(lh.x * sp.fr.tangent + lh.y * sp.fr.bitangent + lh.z * sp.n);
}

// --------------------------------------------------------------- lights ----
__device__ __forceinline__ float lightSelectionCDF(const DevScene& S, uint32_t i) {  // :1546-1548
    return clampf(__ldg(&S.lights[i].selection_cdf), 0.0f, 1.0f);
}
__device__ __forceinline__ float lightSelectionPDF(const DevScene& S, uint32_t i) {  // :1550-1553
    float prev = i == 0u ? 0.0f : lightSelectionCDF(S, i - 1u);
    return fmaxf(lightSelectionCDF(S, i) - prev, 0.0f);
}
__device__ __forceinline__ uint32_t selectLightIndex(const DevScene& S, float sample) {  // :1559-1576
    if (S.light_count <= 1u) return 0u;
    float target = clampf(sample, 0.0f, 0.99999994f);
    uint32_t lo = 0u, hi = S.light_count - 1u;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1u;
        if (target <= lightSelectionCDF(S, mid)) hi = mid; else lo = mid + 1u;
    }
    return lo;
}
__device__ float lightPDFForHit(const DevScene& S, const Hit& h, float3 incoming) {  // :1578-1608
    if (h.primitiveID >= S.tri_count) return 0.0f;
    uint32_t plus1 = __ldg(&S.tris[h.primitiveID].padding2);
    if (plus1 == 0u) return 0.0f;
    uint32_t index = plus1 - 1u;
    if (index >= S.light_count) return 0.0f;
    const dk_light_record& L = S.lights[index];
    float area = __ldg(&L.area);
    if (__ldg(&L.triangle_index) != h.primitiveID || area <= 0.0f) return 0.0f;
    float cosLight = fmaxf(0.0f, dot(xyz(__ldg(reinterpret_cast<const float4*>(&L.normal))), -incoming));
    if (cosLight <= 0.0f) return 0.0f;
    return lightSelectionPDF(S, index) * ((h.t * h.t) / fmaxf(cosLight * area, 1e-6f));
}
__device__ float3 sampleGGXHalfVector(float ux, float uy, float3 n, float roughness) {  // :1610-1618
    float a = roughness * roughness;
    float a2 = a * a;
    float s, c;
    sincosf(6.28318530718f * ux, &s, &c);
    float cosT = sqrtf((1.0f - uy) / fmaxf(1.0f + (a2 - 1.0f) * uy, 1e-5f));
    float sinT = sqrtf(fmaxf(0.0f, 1.0f - cosT * cosT));
    return orientHemisphere(f3(c * sinT, s * sinT, cosT), n);
}
__device__ __forceinline__ float3 sampleTriangle(const dk_triangle& tri, float rx, float ry) {  // :1711-1717
    float su0 = sqrtf(rx);
    float b0 = 1.0f - su0, b1 = su0 * (1.0f - ry), b2 = su0 * ry;
    return b0 * xyz(__ldg(reinterpret_cast<const float4*>(&tri.v0))) +
           b1 * xyz(__ldg(reinterpret_cast<const float4*>(&tri.v1))) +
           b2 * xyz(__ldg(reinterpret_cast<const float4*>(&tri.v2)));
}

// ---------------------------------------------- textures / environment -----
// sampleTexture (:3723-3763) in exact ops, so albedo AOVs stay bit-exact.
__device__ float4 sampleTexture(const DevScene& S, uint32_t plus1, float2 uv, float4 fallback) {
    if (plus1 == 0u || plus1 > S.texdesc_count) return fallback;
    uint4 md = __ldg(reinterpret_cast<const uint4*>(&S.texdesc[plus1 - 1u]));
    uint32_t off = md.x, w = md.y, hgt = md.z, mode = md.w;
    if (w == 0u || hgt == 0u) return fallback;
    float wx = fractf(uv.x), wy = fractf(uv.y);
    if (mode == 1u && w > 1u && hgt > 1u) {
        float tx = ex::sub(ex::mul(wx, (float)w), 0.5f), ty = ex::sub(ex::mul(wy, (float)hgt), 0.5f);
        float bx = floorf(tx), by = floorf(ty);
        float fx = fractf(tx), fy = fractf(ty);
        uint32_t x0 = (uint32_t)fmodf(ex::add(bx, (float)w), (float)w);
        uint32_t y0 = (uint32_t)fmodf(ex::add(by, (float)hgt), (float)hgt);
        uint32_t x1 = (x0 + 1u) % w, y1 = (y0 + 1u) % hgt;
        float4 c00 = __ldg(S.texpix + off + y0 * w + x0), c10 = __ldg(S.texpix + off + y0 * w + x1);
        float4 c01 = __ldg(S.texpix + off + y1 * w + x0), c11 = __ldg(S.texpix + off + y1 * w + x1);
        auto lerp4 = [](float4 a, float4 b, float t) {
            return make_float4(ex::add(a.x, ex::mul(ex::sub(b.x, a.x), t)), ex::add(a.y, ex::mul(ex::sub(b.y, a.y), t)),
                               ex::add(a.z, ex::mul(ex::sub(b.z, a.z), t)), ex::add(a.w, ex::mul(ex::sub(b.w, a.w), t)));
        };
        return lerp4(lerp4(c00, c10, fx), lerp4(c01, c11, fx), fy);
    }
    uint32_t x = min((uint32_t)ex::mul(wx, (float)w), w - 1u);
    uint32_t y = min((uint32_t)ex::mul(wy, (float)hgt), hgt - 1u);
    return __ldg(S.texpix + off + y * w + x);
}
__device__ __forceinline__ float3 fallbackSky(float3 d) {  // :3765-3768
    float sky = 0.5f * (d.y + 1.0f);
    return mix3(f3(0.02f, 0.025f, 0.035f), f3(0.25f, 0.32f, 0.45f), sky);
}
__device__ __forceinline__ float3 rotateEnv(const DevScene& S, float3 d, float& sn, float& cs) {
    sn = S.env_rot_sin;
    cs = S.env_rot_cos;
    return normalize(f3(cs * d.x - sn * d.z, d.y, sn * d.x + cs * d.z));
}
__device__ __forceinline__ float3 sampleEnvironment(const DevScene& S, float3 d) {  // :3770-3802
    float intensity = fmaxf(S.env_intensity, 0.0f);
    if (S.env_tex_plus1 == 0u) return fallbackSky(d) * intensity;
    float sn, cs;
    float3 r = rotateEnv(S, d, sn, cs);
    float u = atan2f(r.z, r.x) * 0.15915494309f + 0.5f;
    float v = clampf(acosf(clampf(r.y, -1.0f, 1.0f)) * 0.31830988618f, 0.00001f, 0.99999f);
    float3 fb = fallbackSky(d);
    float3 color = xyz(sampleTexture(S, S.env_tex_plus1, make_float2(u, v), make_float4(fb.x, fb.y, fb.z, 1.0f))) * intensity;
    float maxR = fmaxf(S.env_max_radiance, 0.0f);
    if (maxR > 0.0f) color = mn(color, f3(maxR));
    return color;
}
__device__ __forceinline__ float environmentPDF(const DevScene& S, float3 d) {  // :3870-3914
    if (S.env == nullptr || S.env_count == 0u || S.env_tex_plus1 == 0u) return 0.0f;
    uint4 md = __ldg(reinterpret_cast<const uint4*>(&S.texdesc[S.env_tex_plus1 - 1u]));
    uint32_t w = md.y, hgt = md.z;
    uint32_t index = 0u;
    if (w != 0u && hgt != 0u) {
        float sn, cs;
        float3 r = rotateEnv(S, d, sn, cs);
        float u = fractf(atan2f(r.z, r.x) * 0.15915494309f + 0.5f);
        float v = clampf(acosf(clampf(r.y, -1.0f, 1.0f)) * 0.31830988618f, 0.0f, 0.99999994f);
        uint32_t x = min((uint32_t)(u * (float)w), w - 1u);
        uint32_t y = min((uint32_t)(v * (float)hgt), hgt - 1u);
        index = y * w + x;
    }
    if (index >= S.env_count) return 0.0f;
    return fmaxf(__ldg(&S.env[index].y), 0.0f);
}
// sampleEnvironmentDirection (:3937-3987) with selectEnvironmentSampleIndex (:3916-3935).
__device__ __forceinline__ float3 sampleEnvironmentDirection(const DevScene& S, float px, float py, float cdfSample, float& pdf) {
    pdf = 0.0f;
    if (S.env_tex_plus1 == 0u || S.env_count == 0u || S.env == nullptr) return f3(0, 1, 0);
    uint4 md = __ldg(reinterpret_cast<const uint4*>(&S.texdesc[S.env_tex_plus1 - 1u]));
    uint32_t w = md.y, hgt = md.z;
    if (w == 0u || hgt == 0u) return f3(0, 1, 0);
    // selectEnvironmentSampleIndex: the first index with target <= cdf[i]
    // (clamped to the last).  The guide table bounds that index for the
    // target's 1/G bucket, so the search covers only the bucket's range and
    // returns the same index as the full binary search over a monotone CDF.
    uint32_t index = 0u;
    if (S.env_count > 1u) {
        float target = clampf(cdfSample, 0.0f, 0.99999994f);
        uint32_t lo = 0u, hi = S.env_count - 1u;
        if (S.env_guide_size) {
            uint32_t bucket = min((uint32_t)(target * (float)S.env_guide_size), S.env_guide_size - 1u);
            lo = min(__ldg(S.env_guide + bucket), S.env_count - 1u);
            hi = min(__ldg(S.env_guide + bucket + 1u), S.env_count - 1u);
        }
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1u;
            if (target <= __ldg(&S.env[mid].x)) hi = mid; else lo = mid + 1u;
        }
        index = lo;
    }
    index = min(index, S.env_count - 1u);
    uint32_t x = index % w, y = index / w;
    float u = ((float)x + px) / (float)w;
    float v = ((float)y + py) / (float)hgt;
    float phi = (u - 0.5f) * 6.28318530718f;
    float theta = clampf(v, 0.00001f, 0.99999f) * 3.14159265359f;
    float sp, cp, st, ct;
    sincosf(phi, &sp, &cp);
    sincosf(theta, &st, &ct);
    float3 local = normalize(f3(cp * st, ct, sp * st));
    float sn = S.env_rot_sin, cs = S.env_rot_cos;
    pdf = fmaxf(__ldg(&S.env[index].y), 0.0f);
    return normalize(f3(cs * local.x + sn * local.z, local.y, -sn * local.x + cs * local.z));
}

}  // namespace dk
