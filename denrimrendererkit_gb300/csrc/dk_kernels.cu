// Wavefront kernels of the sm_103a progressive path tracer.
//
// The reference runs the whole path of a pixel-sample in one thread
// (pathTraceKernel, Sources/DenrimRendererKit/Resources/Shaders/
// PathTrace.metal:5167-5586).  Here one batch of paths (tile pixels x several
// sample indices) advances bounce by bounce through four stages over SoA path
// state in HBM:
//   k_generate  camera rays + RNG seeds              (:5204-5225)
//   k_extend    closest hit of every active ray      (intersectScene, :3294-3421)
//   k_shade     the bounce body: misses, materials, random walks, emission,
//               NEE ray generation, BSDF sampling, Russian roulette  (:5252-5518)
//   k_shadow    the NEE shadow queries and the clamped direct-light sum
//               (sampleDirectLighting, :4407-4585; shadowOccluded, :4196-4274)
//   k_finalize  Kahan-compensated accumulation + last-sample AOVs (:5520-5585)
// Surviving paths are compacted into the next queue with warp-ballot appends.
#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "dk_kernels.h"
#include "dk_sdf.cuh"
#include "dk_shade.cuh"

namespace dk {

__device__ __forceinline__ uint32_t laneId() { return threadIdx.x & 31u; }

// Warp-aggregated append: one atomic per warp, order-stable within the warp.
__device__ __forceinline__ uint32_t warpAppend(uint32_t* counter, bool pred) {
    unsigned active = __activemask();
    unsigned ballot = __ballot_sync(active, pred);
    if (ballot == 0u) return 0u;
    int leader = __ffs(ballot) - 1;
    uint32_t base = 0;
    if ((int)laneId() == leader) base = atomicAdd(counter, (uint32_t)__popc(ballot));
    base = __shfl_sync(active, base, leader);
    unsigned lower = ballot & ((1u << laneId()) - 1u);
    return base + (uint32_t)__popc(lower);
}

// makeCameraRay (PathTrace.metal:4056-4091); pinhole arithmetic in exact ops.
__device__ Ray makeCameraRay(const dk_camera& cam, uint32_t width, uint32_t height, uint32_t gx, uint32_t gy, float jx,
                             float jy, float lx, float ly) {
    float u = ex::div(ex::add((float)gx, jx), (float)width);
    float v = ex::sub(1.0f, ex::div(ex::add((float)gy, jy), (float)height));
    float3 ll = f3(cam.lower_left.x, cam.lower_left.y, cam.lower_left.z);
    float3 hz = f3(cam.horizontal.x, cam.horizontal.y, cam.horizontal.z);
    float3 vt = f3(cam.vertical.x, cam.vertical.y, cam.vertical.z);
    float3 planePoint = ex::add(ex::add(ll, ex::mul(u, hz)), ex::mul(v, vt));
    Ray ray;
    if (cam.origin.w > 0.5f) {
        ray.origin = planePoint;
        ray.direction = ex::normalize(ex::cross(vt, hz));
    } else {
        ray.origin = f3(cam.origin.x, cam.origin.y, cam.origin.z);
        ray.direction = ex::normalize(ex::sub(planePoint, ray.origin));
    }
    float aperture = fmaxf(cam.lens.x, 0.0f);
    if (cam.origin.w <= 0.5f && aperture > 0.0f) {
        float3 forward = normalize(cross(vt, hz));
        float focus = fmaxf(cam.lens.y, 0.0001f);
        float focalT = focus / fmaxf(dot(ray.direction, forward), 0.0001f);
        float3 focal = ray.origin + ray.direction * focalT;
        float2 disk = uniformDisk(lx, ly);
        disk.x *= aperture;
        disk.y *= aperture;
        ray.origin += normalize(hz) * disk.x + normalize(vt) * disk.y;
        ray.direction = normalize(focal - ray.origin);
    }
    return ray;
}

// applyNormalMap (PathTrace.metal:4021-4054).
__device__ Hit applyNormalMap(const DevScene& S, Hit h, uint32_t idx, float3 rayDir) {
    float3 mapped = xyz(sampleTexture(S, idx, h.uv, make_float4(0.5f, 0.5f, 1.0f, 1.0f)));
    mapped = ex::normalize(ex::sub(ex::mul(mapped, 2.0f), f3(1.0f)));
    float3 t = ex::sub(h.tangent, ex::mul(h.normal, ex::dot(h.tangent, h.normal)));
    if (__fsqrt_rn(ex::dot(t, t)) <= 1e-5f) {
        float3 helper = fabsf(h.normal.y) < 0.999f ? f3(0, 1, 0) : f3(1, 0, 0);
        t = ex::cross(helper, h.normal);
    }
    t = ex::normalize(t);
    float3 b = ex::sub(h.bitangent, ex::mul(h.normal, ex::dot(h.bitangent, h.normal)));
    if (__fsqrt_rn(ex::dot(b, b)) <= 1e-5f) b = ex::cross(h.normal, t);
    b = ex::normalize(b);
    h.normal = ex::normalize(ex::add(ex::add(ex::mul(mapped.x, t), ex::mul(mapped.y, b)), ex::mul(mapped.z, h.normal)));
    if (ex::dot(h.normal, rayDir) > 0.0f) h.normal = -h.normal;
    return h;
}

__device__ __forceinline__ float4 exMix4(float4 a, float4 b, float t) {
    return make_float4(exMix(a.x, b.x, t), exMix(a.y, b.y, t), exMix(a.z, b.z, t), exMix(a.w, b.w, t));
}

// blendMaterials (:527-547): m = mix(m, materials[b], t) field by field.
__device__ __noinline__ void blendMaterialInto(Material& m, const dk_material* mats, uint32_t b, float t) {
    const float4* p = reinterpret_cast<const float4*>(mats + b);
    float4* f = reinterpret_cast<float4*>(&m);
#pragma unroll 1
    for (int k = 0; k < 17; ++k) f[k] = exMix4(f[k], __ldg(p + k), t);
}

// A render's material table: S.mats[base, base + count).
struct MatTable {
    uint32_t base, count;
};

__device__ __forceinline__ MatTable matTable(const DevJob& J) {
    return MatTable{__ldg(&J.mat_base), __ldg(&J.mat_count)};
}

// materialForHit (:1096-1121); the material-program VM and the field
// overrides are no-ops here (no programs, no material-field samples).
__device__ __forceinline__ Material materialForHit(const DevScene& S, MatTable mt, const Hit& h) {
    Material m = loadMaterial(S.mats, mt.base + min(h.materialID, mt.count - 1u));
    if (h.materialBlend > 0.0f)
        blendMaterialInto(m, S.mats, mt.base + min(h.materialID2, mt.count - 1u), clampf(h.materialBlend, 0.0f, 1.0f));
    return m;
}

__device__ __forceinline__ VolumeScene volumeScene(const DevScene& S) {
    VolumeScene V;
    V.volumes = S.volumes;
    V.bricks = S.bricks;
    V.samples = S.brick_samples;
    V.dist = DistSrc{S.brick_dist, S.brick_dist16};
    V.grids = S.brick_grids;
    V.gridIndices = S.brick_grid_indices;
    V.sampleCount = S.brick_sample_count;
    V.gridIndexCount = S.brick_grid_index_count;
    V.volumeCount = S.volume_count;
    V.brickCount = S.brick_count;
    V.gridCount = S.brick_grid_count;
    return V;
}

// Hit attributes of a distance-field hit at (t, brick): the tail of
// intersectVolumeBrickPrepared (PathTrace.metal:2741-2802).
__device__ __noinline__ Hit makeVolumeHit(const DevScene& S, const Ray& ray, float t, uint32_t brickIndex) {
    VolumeScene V = volumeScene(S);
    const dk_volume_brick_descriptor& brick = V.bricks[brickIndex];
    uint32_t vi = __ldg(&brick.grid_origin_and_volume.w);
    if (vi >= V.volumeCount) vi = 0;
    const dk_volume_descriptor& vol = V.volumes[vi];
    VolumeRay vr = volumeRay(vol, ray.origin, ray.direction);
    BrickCtx c = makeBrickCtx(brick, V.sampleCount);
    float3 rp = ex::add(vr.lo, ex::mul(vr.ld, t));
    bool cubic = vr.cellSize <= 0.03f;
    Hit h;
    h.t = t;
    h.position = ex::add(ray.origin, ex::mul(ray.direction, t));
    float3 n = brickNormal(V, vol, c, rp, cubic, !cubic);
    h.frontFacing = ex::dot(n, ray.direction) <= 0.0f;
    if (!h.frontFacing) n = -n;
    h.normal = n;
    h.uv = make_float2(0.0f, 0.0f);
    h.tangent = ex::normalize(ex::cross(fabsf(n.y) < 0.999f ? f3(0, 1, 0) : f3(1, 0, 0), n));
    h.bitangent = ex::normalize(ex::cross(n, h.tangent));
    // sampleVolumeBrickMaterial: nearest stored sample (:2319-2372)
    float3 uvw = clamp3(exDiv(ex::sub(rp, c.sampleMin), c.sampleExtent), f3(0.0f), f3(1.0f));
    uint32_t nx = min((uint32_t)roundf(ex::mul(uvw.x, (float)(c.dims[0] - 1u))), c.dims[0] - 1u);
    uint32_t ny = min((uint32_t)roundf(ex::mul(uvw.y, (float)(c.dims[1] - 1u))), c.dims[1] - 1u);
    uint32_t nz = min((uint32_t)roundf(ex::mul(uvw.z, (float)(c.dims[2] - 1u))), c.dims[2] - 1u);
    uint4 ms = __ldg(reinterpret_cast<const uint4*>(V.samples + c.sampleOffset + nx + ny * c.strideY + nz * c.strideZ));
    h.materialID = ms.y;
    h.materialID2 = ms.z;
    h.materialBlend = clampf(__uint_as_float(ms.w), 0.0f, 1.0f);
    h.objectID = __ldg(&vol.metadata.y);
    h.primitiveID = __ldg(&vol.metadata.z);
    return h;
}

__device__ __forceinline__ Hit makeHitAny(const DevScene& S, const Ray& ray, const HitRec& r) {
    if (r.tri == kVolumeHit) return makeVolumeHit(S, ray, r.t, __float_as_uint(r.u));
    return makeHit(S, ray, r);
}

// intersectScene (:3294-3421): triangles, then the sparse volumes with the
// triangle distance as the bound.  traceSceneCounting also counts the volume
// walk's events into the session's SDF traversal counters when it has them;
// the subsurface walk inside the shading kernel takes the plain form, which
// keeps that kernel's registers (its walk steps still count as scene queries).
__device__ __noinline__ HitRec traceScene(const DevScene& S, float3 o, float3 d) {
    HitRec r = S.wide8 ? traceClosest8(S, o, d) : traceClosest(S, o, d);
    if (S.volume_count) {
        VolumeHitRec vh;
        if (closestVolumeHit(volumeScene(S), o, d, r.t, vh)) {
            r.t = vh.t;
            r.tri = kVolumeHit;
            r.u = __uint_as_float(vh.brick);
            r.v = 0.0f;
        }
    }
    return r;
}
__device__ __noinline__ HitRec traceSceneCounting(const DevScene& S, float3 o, float3 d) {
    HitRec r = S.wide8 ? traceClosest8(S, o, d) : traceClosest(S, o, d);
    if (S.volume_count) {
        VolumeHitRec vh;
        if (closestVolumeHitAny(volumeScene(S), o, d, r.t, vh, S.sdf_counters)) {
            r.t = vh.t;
            r.tri = kVolumeHit;
            r.u = __uint_as_float(vh.brick);
            r.v = 0.0f;
        }
    }
    return r;
}

// Subsurface walk helpers (PathTrace.metal:3490-3523).
__device__ __forceinline__ float sampleSubsurfaceFreeFlight(float3 sigmaT, float ux, float uy) {
    float sigma = sigmaT.z;
    if (ux < 0.33333333333f) sigma = sigmaT.x;
    else if (ux < 0.66666666667f) sigma = sigmaT.y;
    return -logf(fmaxf(1.0f - uy, 1e-6f)) / fmaxf(sigma, 1e-4f);
}
__device__ __forceinline__ float subsurfaceCollisionPDF(float3 s, float d) {
    float3 tr = exp3((-s) * d);
    return fmaxf((s.x * tr.x + s.y * tr.y + s.z * tr.z) * 0.33333333333f, 1e-6f);
}
__device__ __forceinline__ float subsurfaceBoundaryPDF(float3 s, float d) {
    float3 tr = exp3((-s) * d);
    return fmaxf((tr.x + tr.y + tr.z) * 0.33333333333f, 1e-6f);
}

// continueSubsurfaceRandomWalk (PathTrace.metal:3525-3621).
template <bool kVolumes>
__device__ bool continueSubsurfaceRandomWalk(const DevScene& S, const Hit& entry, const Material& m, Ray& ray,
                                             float3& tp, float& prevPdf, uint32_t& state) {
    if (materialSubsurface(m) <= 0.0f || !entry.frontFacing) return false;
    float e0 = randomFloat(state);
    float e1 = randomFloat(state);
    float3 entryDir = orientHemisphere(cosineHemisphere(e0, e1), -entry.normal);
    Ray medium{entry.position + entryDir * 0.001f, entryDir};
    float3 sigmaT = 1.0f / mx(xyz(m.subsurfaceRadius) * fmaxf(m.subsurfaceRadius.w, 0.0f), f3(1e-4f));
    float3 albedo = clamp3(xyz(m.subsurfaceColor), f3(0.0f), f3(0.999f));
    float anisotropy = clampf(m.subsurfaceParameters.x, -0.95f, 0.95f);
    for (uint32_t step = 0u; step < 8u; ++step) {
        sdfCount(S.sdf_counters, kSdfBounceSceneQueries);
        HitRec r = kVolumes ? traceScene(S, medium.origin, medium.direction) : traceClosest(S, medium.origin, medium.direction);
        if (r.tri == kNoHit) return false;
        float f0 = randomFloat(state);
        float f1 = randomFloat(state);
        float freeFlight = sampleSubsurfaceFreeFlight(sigmaT, f0, f1);
        if (freeFlight < r.t) {
            medium.origin += medium.direction * freeFlight;
            float h0 = randomFloat(state);
            float h1 = randomFloat(state);
            medium.direction = sampleHenyeyGreenstein(h0, h1, medium.direction, anisotropy);
            float3 tr = exp3((-sigmaT) * freeFlight);
            tp *= albedo * sigmaT * tr / subsurfaceCollisionPDF(sigmaT, freeFlight);
            if (maxComponent(tp) <= 1e-4f) return false;
            continue;
        }
        Hit b = kVolumes ? makeHitAny(S, medium, r) : makeHit(S, medium, r);
        float3 exitNormal = normalize(b.frontFacing ? b.normal : -b.normal);
        float x0 = randomFloat(state);
        float x1 = randomFloat(state);
        ray.direction = orientHemisphere(cosineHemisphere(x0, x1), exitNormal);
        ray.origin = b.position + exitNormal * 0.001f;
        float3 tr = exp3((-sigmaT) * r.t);
        tp *= tr / subsurfaceBoundaryPDF(sigmaT, r.t);
        prevPdf = fmaxf(dot(exitNormal, ray.direction), 0.0f) * 0.31830988618f;
        return true;
    }
    return false;
}

// continueTransmissionVolumeRandomWalk (PathTrace.metal:3685-3721).
__device__ bool continueTransmissionVolumeRandomWalk(const Hit& b, const Material& m, Ray& ray, float3& tp,
                                                     float& prevPdf, uint32_t& state) {
    if (b.frontFacing || !materialHasVolumeScattering(m)) return false;
    float3 sigmaT = materialVolumeSigmaT(m);
    float3 sigmaS = materialVolumeSigmaS(m);
    if (maxComponent(sigmaT) <= 1e-5f || maxComponent(sigmaS) <= 1e-5f) return false;
    float f0 = randomFloat(state);
    float f1 = randomFloat(state);
    float freeFlight = sampleSubsurfaceFreeFlight(sigmaT, f0, f1);
    if (freeFlight >= b.t) {
        tp *= exp3((-sigmaT) * b.t) / subsurfaceBoundaryPDF(sigmaT, b.t);
        return false;
    }
    float3 tr = exp3((-sigmaT) * freeFlight);
    tp *= sigmaS * tr / subsurfaceCollisionPDF(sigmaT, freeFlight);
    ray.origin += ray.direction * freeFlight;
    float h0 = randomFloat(state);
    float h1 = randomFloat(state);
    ray.direction = sampleHenyeyGreenstein(h0, h1, ray.direction, clampf(m.volumeParameters.y, -0.95f, 0.95f));
    ray.origin += ray.direction * 0.001f;
    prevPdf = 0.0f;
    return maxComponent(tp) > 1e-4f;
}

// continueTransmissiveSurface (PathTrace.metal:1723-1799).
__device__ bool continueTransmissiveSurface(const Hit& h, const Material& m, Ray& ray, float3& tp, float& prevPdf,
                                            uint32_t& state) {
    float transmission = materialTransmission(m);
    if (transmission <= 0.0f || randomFloat(state) > transmission) return false;
    float3 incoming = ray.direction;
    float3 view = -incoming;
    float roughness = clampf(m.parameters3.y, 0.001f, 1.0f);
    float ior = fmaxf(m.parameters3.z, 1.0001f);
    float3 micro = h.normal;
    if (roughness > 0.01f) {
        float a = randomFloat(state);
        float b = randomFloat(state);
        micro = sampleGGXHalfVector(a, b, h.normal, roughness);
        if (dot(micro, incoming) > 0.0f) micro = -micro;
    }
    float etaI = h.frontFacing ? 1.0f : ior;
    float etaT = h.frontFacing ? ior : 1.0f;
    float eta = etaI / etaT;
    float cosI = fmaxf(dot(view, micro), 0.0f);
    float fresnel = dielectricFresnel(cosI, etaI, etaT);
    if (materialThinWalled(m)) {
        fresnel = dielectricFresnel(cosI, 1.0f, ior);
        float rp = clampf(fresnel, 0.02f, 0.98f);
        if (randomFloat(state) < rp) {
            ray.direction = normalize(reflect(incoming, micro));
            ray.origin = h.position + micro * 0.001f;
            tp *= fresnel / fmaxf(rp, 1e-5f);
        } else {
            ray.direction = incoming;
            ray.origin = h.position + ray.direction * 0.001f;
            float grazing = 1.0f - fabsf(dot(view, h.normal));
            float tint = mixf(0.35f, 0.95f, grazing * grazing);
            tp *= materialTransmissionTint(m, tint) * ((1.0f - fresnel) / fmaxf(1.0f - rp, 1e-5f));
        }
        prevPdf = 0.0f;
        return true;
    }
    float3 refracted = refract(incoming, micro, eta);
    bool tir = dot(refracted, refracted) <= 1e-7f;
    float rp = tir ? 1.0f : clampf(fresnel, 0.02f, 0.98f);
    if (randomFloat(state) < rp) {
        ray.direction = normalize(reflect(incoming, micro));
        ray.origin = h.position + micro * 0.001f;
        tp *= tir ? 1.0f : fresnel / fmaxf(rp, 1e-5f);
    } else {
        ray.direction = normalize(refracted);
        ray.origin = h.position + ray.direction * 0.001f;
        float grazing = 1.0f - fabsf(dot(view, h.normal));
        float tint = mixf(0.35f, 0.95f, grazing * grazing);
        float w = (1.0f - fresnel) / fmaxf(1.0f - rp, 1e-5f);
        float3 absorption = materialTransmissionAbsorption(m, h.t, !h.frontFacing && !materialHasVolumeScattering(m));
        tp *= materialTransmissionTint(m, tint) * absorption * w;
    }
    prevPdf = 0.0f;
    return true;
}

// ================================================================ kernels ==

__device__ __forceinline__ uint32_t gridStride() { return gridDim.x * blockDim.x; }
__device__ __forceinline__ uint32_t globalId() { return blockIdx.x * blockDim.x + threadIdx.x; }

// The job whose [begin, next begin) range holds `i` (the last job whose
// begin <= i), by binary search over the wave's ascending job table.
__device__ __forceinline__ uint32_t jobOfPath(const Wave& W, uint32_t i) {
    uint32_t lo = 0, hi = W.job_count - 1u;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1u) >> 1;
        if (__ldg(&W.jobs[mid].path_begin) <= i) lo = mid; else hi = mid - 1u;
    }
    return lo;
}
__device__ __forceinline__ uint32_t jobOfPixel(const Wave& W, uint32_t i) {
    uint32_t lo = 0, hi = W.job_count - 1u;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1u) >> 1;
        if (__ldg(&W.jobs[mid].pixel_begin) <= i) lo = mid; else hi = mid - 1u;
    }
    return lo;
}
__device__ __forceinline__ uint32_t jobOf(const Wave& W, uint32_t p) { return W.rng[p].y >> 8; }

__device__ __forceinline__ void writeAovMiss(float4* aov, uint32_t local, uint32_t tileN) {
    aov[0 * (size_t)tileN + local] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(0u));  // t, -, -, hasHit
    aov[1 * (size_t)tileN + local] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    aov[2 * (size_t)tileN + local] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    aov[3 * (size_t)tileN + local] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}
__device__ __forceinline__ void writeAovHit(float4* aov, uint32_t local, uint32_t tileN, const Hit& h, float4 albedo) {
    aov[0 * (size_t)tileN + local] = make_float4(h.t, __uint_as_float(h.materialID), __uint_as_float(h.objectID), __uint_as_float(1u));
    aov[1 * (size_t)tileN + local] = make_float4(h.normal.x, h.normal.y, h.normal.z, 0.0f);
    aov[2 * (size_t)tileN + local] = albedo;
    aov[3 * (size_t)tileN + local] = make_float4(h.position.x, h.position.y, h.position.z, 0.0f);
}

__global__ void __launch_bounds__(256) k_generate(DevScene S, Wave W) {
    for (uint32_t p = globalId(); p < W.path_count; p += gridStride()) {
        uint32_t j = jobOfPath(W, p);
        const DevJob& J = W.jobs[j];
        const DevParams& P = J.P;
        const uint32_t tileN = P.tile_w * P.tile_h;
        uint32_t rel = p - J.path_begin;
        uint32_t slice = rel / tileN, local = rel - slice * tileN;
        uint32_t px = P.tile_x + local % P.tile_w, py = P.tile_y + local / P.tile_w;
        uint32_t sample = P.sample_begin + slice;
        uint32_t state = P.frame_seed ^ hash_u32(px + py * P.width) ^ hash_u32(sample + 1u);
        float j0 = randomFloat(state);
        float j1 = randomFloat(state);
        float j2 = randomFloat(state);
        float j3 = randomFloat(state);
        Ray ray = makeCameraRay(P.cam, P.width, P.height, px, py, j0, j1, j2, j3);
        W.ray_o[p] = make_float4(ray.origin.x, ray.origin.y, ray.origin.z, 0.0f);
        W.ray_d[p] = make_float4(ray.direction.x, ray.direction.y, ray.direction.z, 0.0f);
        W.tp[p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        W.rad[p] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        W.rng[p] = make_uint2(state, j << 8);
        W.q[0][p] = p;
        if (slice == P.samples_in_batch - 1u) writeAovMiss(W.aov, J.pixel_begin + local, W.aov_stride);
    }
    if (globalId() == 0) {
        W.counts[0] = W.path_count;
        for (int k = 1; k < 8; ++k) W.counts[k] = 0u;
    }
}

constexpr uint32_t kNoWork = 0xffffffffu;
#ifndef DK_STEP_BUDGET
#define DK_STEP_BUDGET 16
#endif
constexpr int kStepBudget = DK_STEP_BUDGET;

// Refills the lanes that asked for work with consecutive items of a queue of
// length `n` through one atomic per warp; returns this lane's item or kNoWork.
__device__ __forceinline__ uint32_t warpFetch(uint32_t* counter, uint32_t n, bool need, bool& exhausted) {
    unsigned m = __ballot_sync(0xffffffffu, need);
    if (m == 0u) return kNoWork;
    int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if ((int)laneId() == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (!need) return kNoWork;
    uint32_t idx = base + (uint32_t)__popc(m & ((1u << laneId()) - 1u));
    if (idx >= n) {
        exhausted = true;
        return kNoWork;
    }
    return idx;
}

// Closest hit for every ray of the input queue (intersectScene), persistent
// threads with per-lane refill.  W.counts[4] is the work cursor (zeroed by the
// kernel that runs before).
template <bool kWide8>
__global__ void __launch_bounds__(128) k_extend(DevScene S, Wave W, uint32_t sel, uint32_t bounce) {
    const uint32_t* q = W.q[sel];
    const uint32_t n = W.counts[sel];
    if (blockIdx.x == 0)
        for (uint32_t b = threadIdx.x; b <= kSortBins; b += blockDim.x) W.bins[b] = 0u;
    if (globalId() == 0) {
        // one scene query per active path and bounce (PathTrace.metal:5252-5256)
        if (S.sdf_counters && n)
            atomicAdd(S.sdf_counters + (bounce == 0u ? kSdfPrimarySceneQueries : kSdfBounceSceneQueries),
                      (unsigned long long)n);
        W.counts[sel ^ 1u] = 0u;
        W.counts[2] = 0u;
        W.counts[3] = 0u;
        W.counts[5] = 0u;
        W.counts[6] = 0u;
        W.counts[7] = 0u;
        W.counts[8] = 0u;
    }
    // The stacks stay separate objects from the scalar state, so that only
    // they live in local memory.
    int stackNode[kWide8 ? 1 : kStackSize];
    float stackT[kWide8 ? 1 : kStackSize];
    uint2 stack8[kWide8 ? kTraversalStack : 1];
    std::conditional_t<kWide8, Closest8, ClosestState> st;
    uint32_t p = kNoWork;
    bool exhausted = false;
    for (;;) {
        uint32_t idx = warpFetch(&W.counts[4], n, p == kNoWork && !exhausted, exhausted);
        if (idx != kNoWork) {
            p = q[idx];
            float4 o = W.ray_o[p], d = W.ray_d[p];
            closestInit(st, xyz(o), xyz(d));
            if (S.node_count == 0) {
                W.hit[p] = make_float4(INFINITY, __uint_as_float(kNoHit), 0.0f, 0.0f);
                p = kNoWork;
            }
        }
        if (__all_sync(0xffffffffu, p == kNoWork && exhausted)) break;
        bool done = false;
        if (p != kNoWork) {
            if constexpr (kWide8)
                done = closestSteps(S, st, stack8, kStepBudget);
            else
                done = closestSteps(S, st, stackNode, stackT, kStepBudget);
        }
        if (done) {
            W.hit[p] = make_float4(st.bestT, __uint_as_float(st.bestTri), st.bu, st.bv);
            p = kNoWork;
        }
    }
}

// ------------------------------------------------ material ordering ----
// The active queue is reordered by material before shading (a counting sort
// on the hit's material ID), so the paths of a warp take the same BSDF
// branches and read the same material record.  The order of paths does not
// change any result: every path carries its own RNG state and pixel samples
// are accumulated in sample order.
// Keys: 0 a miss, 1 + material ID (at most kSortBins - 3), kSortBins - 2 a
// material with a subsurface weight (shaded by the kernel that carries the
// subsurface random walk), kSortBins - 1 a distance-volume hit.
constexpr uint32_t kSubsurfaceKey = kSortBins - 2u;
__device__ __forceinline__ uint32_t shadeKey(const DevScene& S, const Wave& W, uint32_t p) {
    uint32_t tri = __float_as_uint(W.hit[p].y);
    if (tri == kNoHit) return 0u;
    if (tri >= S.tri_count) return kSortBins - 1u;  // distance-volume hits
    const uint32_t id = __ldg(&S.tris[tri].material_id);
    // the material the shading kernel loads, and materialSubsurface's own test
    const MatTable mt = matTable(W.jobs[W.rng[p].y >> 8]);
    const float4* q = reinterpret_cast<const float4*>(S.mats + mt.base + min(id, mt.count - 1u));
    Material m;
    m.emission = __ldg(q + 1);
    m.parameters = __ldg(q + 2);
    m.subsurfaceColor = __ldg(q + 12);
    if (materialSubsurface(m) > 0.0f) return kSubsurfaceKey;
    return 1u + min(id, kSortBins - 3u);
}

__global__ void __launch_bounds__(256) k_sort_count(DevScene S, Wave W, uint32_t sel) {
    __shared__ uint32_t hist[kSortBins];
    for (uint32_t b = threadIdx.x; b < kSortBins; b += blockDim.x) hist[b] = 0u;
    __syncthreads();
    const uint32_t* q = W.q[sel];
    const uint32_t n = W.counts[sel];
    for (uint32_t i = globalId(); i < n; i += gridStride()) {
        uint32_t k = shadeKey(S, W, q[i]);
        W.keys[i] = k;
        atomicAdd(&hist[k], 1u);
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < kSortBins; b += blockDim.x)
        if (hist[b]) atomicAdd(&W.bins[b], hist[b]);
}

// Exclusive scan of the histogram into bucket cursors (one block of kSortBins threads).
__global__ void __launch_bounds__(kSortBins) k_sort_scan(Wave W) {
    __shared__ uint32_t v[kSortBins];
    uint32_t t = threadIdx.x;
    uint32_t x = W.bins[t];
    v[t] = x;
    __syncthreads();
    for (uint32_t o = 1; o < kSortBins; o <<= 1) {
        uint32_t y = t >= o ? v[t - o] : 0u;
        __syncthreads();
        v[t] += y;
        __syncthreads();
    }
    W.bins[t] = v[t] - x;
    if (t == kSubsurfaceKey) W.counts[7] = v[t] - x;  // shading-order index of the first subsurface path
}

// Block b places queue entries [b * 2048, b * 2048 + 2048) stably: an entry's
// rank among the block's entries of its key follows queue order (in-warp
// ranks from __match_any_sync, warp offsets per key scanned in shared memory,
// eight rounds of 256 entries in order), and one global reservation per
// (block, key) places the block's run.  The queue is in path order, so every
// run of a key holds increasing path indices -- neighbouring lanes of the
// shading kernel read neighbouring path state.
constexpr uint32_t kSortItems = 8;
__global__ void __launch_bounds__(256) k_sort_scatter(Wave W, uint32_t sel) {
    __shared__ uint32_t cnt[kSortBins];
    __shared__ uint32_t base[kSortBins];
    __shared__ uint32_t warpCnt[8][kSortBins];
    const uint32_t* q = W.q[sel];
    const uint32_t n = W.counts[sel];
    const uint32_t start = blockIdx.x * 256u * kSortItems;
    if (start >= n) return;  // uniform over the block
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t lanesBelow = (1u << lane) - 1u;
    cnt[tid] = 0u;  // kSortBins == blockDim.x
    uint32_t key[kSortItems], rank[kSortItems];
#pragma unroll
    for (uint32_t k = 0; k < kSortItems; ++k) {
#pragma unroll
        for (uint32_t w = 0; w < 8u; ++w) warpCnt[w][tid] = 0u;
        __syncthreads();
        const uint32_t i = start + k * 256u + tid;
        const bool valid = i < n;
        key[k] = valid ? W.keys[i] : kSortBins - 1u;
        const uint32_t peers = __match_any_sync(0xffffffffu, valid ? key[k] : 0xffffffffu);
        const uint32_t inWarp = __popc(peers & lanesBelow);
        if (valid && inWarp == 0u) warpCnt[warp][key[k]] = __popc(peers);
        __syncthreads();
        {  // thread `tid` scans key `tid` over the warps, after the earlier rounds
            uint32_t run = cnt[tid];
#pragma unroll
            for (uint32_t w = 0; w < 8u; ++w) {
                const uint32_t c = warpCnt[w][tid];
                warpCnt[w][tid] = run;
                run += c;
            }
            cnt[tid] = run;
        }
        __syncthreads();
        rank[k] = valid ? warpCnt[warp][key[k]] + inWarp : 0u;
        __syncthreads();
    }
    if (cnt[tid]) base[tid] = atomicAdd(&W.bins[tid], cnt[tid]);
    __syncthreads();
#pragma unroll
    for (uint32_t k = 0; k < kSortItems; ++k) {
        uint32_t i = start + k * 256u + tid;
        if (i < n) W.qsorted[base[key[k]] + rank[k]] = q[i];
    }
}

// ------------------------------------------ survivors in path order ----
// Shading writes a flag per path; the next bounce's queue is the flagged
// paths in increasing path order: a count per block of kLiveBlock paths, one
// block's scan of the counts, and a scatter of each block's paths at its
// offset.  Path order keeps the extension stage's and (through the stable
// material sort) the shading stage's path-state accesses coalesced.
__device__ __forceinline__ uint32_t liveCount16(const Wave& W, uint32_t first, uint32_t n, uint32_t& bits) {
    bits = 0u;
    if (first + 16u <= n) {
        const uint4 v = *reinterpret_cast<const uint4*>(W.live + first);
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (uint32_t j = 0; j < 4u; ++j)
#pragma unroll
            for (uint32_t b = 0; b < 4u; ++b) bits |= (((w[j] >> (8u * b)) & 0xffu) ? 1u : 0u) << (4u * j + b);
    } else {
        for (uint32_t j = 0; j < 16u && first + j < n; ++j) bits |= (W.live[first + j] ? 1u : 0u) << j;
    }
    return __popc(bits);
}

__device__ __forceinline__ uint32_t blockExclusiveScan256(uint32_t v, uint32_t& total) {
    __shared__ uint32_t warpSums[8];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (uint32_t o = 1; o < 32u; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31u) warpSums[warp] = x;
    __syncthreads();
    uint32_t before = 0u;
    total = 0u;
#pragma unroll
    for (uint32_t w = 0; w < 8u; ++w) {
        const uint32_t c = warpSums[w];
        if (w < warp) before += c;
        total += c;
    }
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(256) k_live_count(Wave W) {
    const uint32_t n = W.path_count;
    const uint32_t first = blockIdx.x * kLiveBlock + threadIdx.x * 16u;
    uint32_t bits, total;
    const uint32_t c = first < n ? liveCount16(W, first, n, bits) : 0u;
    blockExclusiveScan256(c, total);
    if (threadIdx.x == 0) W.scan[blockIdx.x] = total;
}

// Exclusive scan of the block counts (one block); the total is the next queue's length.
__global__ void __launch_bounds__(256) k_live_scan(Wave W, uint32_t sel, uint32_t blocks) {
    const uint32_t per = (blocks + 255u) / 256u;
    const uint32_t b0 = threadIdx.x * per;
    uint32_t sum = 0u;
    for (uint32_t b = b0; b < b0 + per && b < blocks; ++b) sum += W.scan[b];
    uint32_t total;
    uint32_t run = blockExclusiveScan256(sum, total);
    for (uint32_t b = b0; b < b0 + per && b < blocks; ++b) {
        const uint32_t c = W.scan[b];
        W.scan[b] = run;
        run += c;
    }
    if (threadIdx.x == 0) W.counts[sel ^ 1u] = total;
}

__global__ void __launch_bounds__(256) k_live_scatter(Wave W, uint32_t sel) {
    const uint32_t n = W.path_count;
    const uint32_t first = blockIdx.x * kLiveBlock + threadIdx.x * 16u;
    uint32_t bits = 0u, total;
    const uint32_t c = first < n ? liveCount16(W, first, n, bits) : 0u;
    uint32_t slot = W.scan[blockIdx.x] + blockExclusiveScan256(c, total);
    uint32_t* qNext = W.q[sel ^ 1u];
    while (bits) {
        const uint32_t j = __ffs(bits) - 1u;
        bits &= bits - 1u;
        qNext[slot++] = first + j;
    }
}

struct ShadeOut { bool survive; uint32_t neeMask; uint32_t maxBounces; };

// The body of the reference bounce loop (PathTrace.metal:5252-5518) for one
// path whose closest hit is already in W.hit.
// kSss: the subsurface random walk is compiled in (the kernel for materials
// with a subsurface weight, and for unsorted queues); without it the walk's
// test is false at compile time, which leaves every other material's path
// as it was (the walk is entered only for a positive weight).
template <bool kVolumes, bool kSss>
__device__ ShadeOut shadePath(const DevScene& S, const Wave& W, uint32_t p, uint32_t i, uint32_t bounce) {
    float4 ro = W.ray_o[p], rd = W.ray_d[p], tpw = W.tp[p], radw = W.rad[p], hr = W.hit[p];
    uint2 rs = W.rng[p];
    const DevJob& J = W.jobs[rs.y >> 8];
    const DevParams& P = J.P;
    ShadeOut out{false, 0u, P.max_bounces};
    Ray ray{xyz(ro), xyz(rd)};
    float3 tp = xyz(tpw);
    float prevPdf = tpw.w;
    float3 rad = xyz(radw);
    float alpha = radw.w;
    uint32_t state = rs.x, flags = rs.y;
    bool primaryFound = (flags & 1u) != 0u;
    uint32_t tri = __float_as_uint(hr.y);

    if (tri == kNoHit) {  // :5279-5305
        if (P.transparent_background != 0u && !primaryFound) {
            alpha = 0.0f;
        } else if (P.shows_env_bg == 0u && !primaryFound) {
            alpha = 1.0f;
            rad += mx(f3(P.bg[0], P.bg[1], P.bg[2]), f3(0.0f));
        } else {
            float envWeight = 1.0f;
            if (bounce > 0u && prevPdf > 0.0f) envWeight = powerHeuristic(prevPdf, environmentPDF(S, ray.direction));
            rad += clampSampleContribution(tp * sampleEnvironment(S, ray.direction) * envWeight, P.clamp);
        }
        W.rad[p] = make_float4(rad.x, rad.y, rad.z, alpha);
        return out;
    }
    HitRec rec{hr.x, tri, hr.z, hr.w};
    Hit h = kVolumes ? makeHitAny(S, ray, rec) : makeHit(S, ray, rec);
    const MatTable mt = matTable(J);
    Material m = kVolumes ? materialForHit(S, mt, h) : loadMaterial(S.mats, mt.base + min(h.materialID, mt.count - 1u));
    uint32_t nIdx = (uint32_t)m.parameters.w;
    if (nIdx != 0u) h = applyNormalMap(S, h, nIdx, ray.direction);
    uint32_t bIdx = (uint32_t)m.parameters.z;
    if (bIdx != 0u) {
        float4 texel = sampleTexture(S, bIdx, h.uv, make_float4(1.0f, 1.0f, 1.0f, 1.0f));
        m.baseColor = make_float4(ex::mul(m.baseColor.x, texel.x), ex::mul(m.baseColor.y, texel.y),
                                  ex::mul(m.baseColor.z, texel.z), ex::mul(m.baseColor.w, texel.w));
    }
    if (m.baseColor.w <= 0.001f) {  // cut-out: pass through (:5318-5321)
        ray.origin = ex::add(h.position, ex::mul(ray.direction, 0.001f));
        W.ray_o[p] = make_float4(ray.origin.x, ray.origin.y, ray.origin.z, 0.0f);
        out.survive = true;
        return out;
    }
    if (!primaryFound) {
        flags |= 1u;
        const uint32_t tileN = P.tile_w * P.tile_h;
        uint32_t rel = p - J.path_begin;
        uint32_t slice = rel / tileN;
        if (slice == P.samples_in_batch - 1u && P.denoiser == 0u)
            writeAovHit(W.aov, J.pixel_begin + (rel - slice * tileN), W.aov_stride, h, m.baseColor);
    }

    bool continued = false;
    if (continueTransmissionVolumeRandomWalk(h, m, ray, tp, prevPdf, state)) {
        continued = true;
    } else {
        float subsurface = materialSubsurface(m);
        if (kSss && subsurface > 0.0f && randomFloat(state) < subsurface &&
            continueSubsurfaceRandomWalk<kVolumes>(S, h, m, ray, tp, prevPdf, state)) {
            continued = true;
        } else if (continueTransmissiveSurface(h, m, ray, tp, prevPdf, state)) {
            continued = true;
        }
    }
    if (continued) {
        bool dead = terminatePathWithRussianRoulette(bounce, tp, state);
        W.ray_o[p] = make_float4(ray.origin.x, ray.origin.y, ray.origin.z, 0.0f);
        W.ray_d[p] = make_float4(ray.direction.x, ray.direction.y, ray.direction.z, 0.0f);
        W.tp[p] = make_float4(tp.x, tp.y, tp.z, prevPdf);
        W.rng[p] = make_uint2(state, flags);
        out.survive = !dead;
        return out;
    }

    float3 emission = xyz(m.emission);
    if (maxComponent(emission) > 0.0f) {  // :5376-5392
        float w = 1.0f;
        if (bounce > 0u && prevPdf > 0.0f) w = powerHeuristic(prevPdf, lightPDFForHit(S, h, ray.direction));
        rad += clampSampleContribution(tp * emission * w, P.clamp);
        W.rad[p] = make_float4(rad.x, rad.y, rad.z, alpha);
        return out;
    }

    // ------------------------------------ NEE (sampleDirectLighting) ------
    float3 view = -ray.direction;
    ShadePoint sp;
    makeShadePoint(sp, m, h.normal, h.tangent, h.bitangent, view);
    float3 shadowOrigin = h.position + h.normal * 0.001f;
    const size_t cap = W.cap;
    // NEE slots are indexed by shading order `i` (coalesced); the slot's
    // direction.w carries the path's job, nee_tp.w the slot mask | path << 3.
    const float jobBits = __uint_as_float(rs.y >> 8);
    if (S.light_count > 0u) {
        uint32_t index = selectLightIndex(S, randomFloat(state));
        const dk_light_record& L = S.lights[index];
        float selPdf = lightSelectionPDF(S, index);
        uint32_t lti = __ldg(&L.triangle_index);
        if (lti < S.tri_count && selPdf > 0.0f) {
            uint32_t lmi = min(__ldg(&L.material_index), S.mat_count - 1u);
            float3 le = xyz(__ldg(reinterpret_cast<const float4*>(S.mats + lmi) + 1));
            float area = __ldg(&L.area);
            if (area > 0.0f) {
                float r0 = randomFloat(state);
                float r1 = randomFloat(state);
                float3 lp = sampleTriangle(S.tris[lti], r0, r1);
                float3 toL = lp - h.position;
                float d2 = dot(toL, toL);
                float dist = sqrtf(d2);
                float3 ld = toL / dist;
                float cosS = fmaxf(0.0f, dot(h.normal, ld));
                float cosL = fmaxf(0.0f, dot(xyz(__ldg(reinterpret_cast<const float4*>(&L.normal))), -ld));
                if (cosS > 0.0f && cosL > 0.0f) {
                    float lightPdf = selPdf * (d2 / fmaxf(cosL * area, 1e-6f));
                    float bsdfPdf = bsdfPDF(sp, ld);
                    float mis = powerHeuristic(lightPdf, bsdfPdf);
                    float G = cosS * cosL * area / fmaxf(d2, 1e-6f);
                    float3 c = evalBRDF(m, sp, ld) * le * G * mis;
                    if (!(c.x == 0.0f && c.y == 0.0f && c.z == 0.0f)) {
                        W.nee_o[i] = make_float4(shadowOrigin.x, shadowOrigin.y, shadowOrigin.z, dist - 0.002f);
                        W.nee_d[i] = make_float4(ld.x, ld.y, ld.z, jobBits);
                        W.nee_c[i] = make_float4(c.x, c.y, c.z, selPdf);
                        out.neeMask |= 1u;
                    }
                }
            }
        }
    }
#pragma unroll 1
    for (uint32_t e = 0u; e < 2u; ++e) {
        float a = randomFloat(state);
        float b = randomFloat(state);
        float cdf = randomFloat(state);
        float envPdf;
        float3 dir = sampleEnvironmentDirection(S, a, b, cdf, envPdf);
        float cosS = fmaxf(0.0f, dot(h.normal, dir));
        if (envPdf > 0.0f && cosS > 0.0f) {
            float bsdfPdf = bsdfPDF(sp, dir);
            float mis = powerHeuristic(envPdf, bsdfPdf);
            float3 c = evalBRDF(m, sp, dir) * sampleEnvironment(S, dir) * cosS * mis;
            if (!(c.x == 0.0f && c.y == 0.0f && c.z == 0.0f)) {
                size_t slot = (size_t)(1u + e) * cap + i;
                W.nee_o[slot] = make_float4(shadowOrigin.x, shadowOrigin.y, shadowOrigin.z, 1.0e20f);
                W.nee_d[slot] = make_float4(dir.x, dir.y, dir.z, jobBits);
                W.nee_c[slot] = make_float4(c.x, c.y, c.z, envPdf * 2.0f);
                out.neeMask |= 2u << e;
            }
        }
    }
    if (out.neeMask) W.nee_tp[i] = make_float4(tp.x, tp.y, tp.z, __uint_as_float(out.neeMask | (p << 3)));

    // --------------------------------------------- BSDF sampling ----------
    float c0 = randomFloat(state);
    float c1 = randomFloat(state);
    float3 diffuseDir = orientHemisphere(cosineHemisphere(c0, c1), h.normal);
    float lobe = randomFloat(state);
    float3 next;
    if (lobe < sp.cP) {
        float a = randomFloat(state);
        float b = randomFloat(state);
        float3 hv = sampleVNDF(sp, a, b, sp.ccAlpha);
        next = normalize(reflect(ray.direction, hv));
        if (dot(next, h.normal) <= 0.0f) {
            next = diffuseDir;
            tp *= diffuseBounceWeight(m, sp, next) / fmaxf(sp.dP, 1e-5f);
        } else {
            float nDotL = fmaxf(dot(h.normal, next), 1e-5f);
            float vDotH = fmaxf(dot(view, hv), 1e-5f);
            tp *= sp.clearcoat * fresnelSchlickThinFilm(vDotH, sp.ccF0, m) * geometrySmithG1GGX(nDotL, sp.ccR) /
                  fmaxf(sp.cP, 1e-5f);
        }
    } else if (lobe < sp.cP + sp.sP) {
        float a = randomFloat(state);
        float b = randomFloat(state);
        float3 hv = sampleVNDF(sp, a, b, sp.specAlpha);
        next = normalize(reflect(ray.direction, hv));
        if (dot(next, h.normal) <= 0.0f) {
            next = diffuseDir;
            tp *= diffuseBounceWeight(m, sp, next) / fmaxf(sp.dP, 1e-5f);
        } else {
            float vDotH = fmaxf(dot(view, hv), 1e-5f);
            float3 fres = fresnelSchlickThinFilm(vDotH, sp.f0, m);
            float3 cca = materialClearcoatAttenuationForDirection(m, h.normal, view, next);
            // The reference passes the raw tangent / bitangent here (PathTrace.metal:5486-5493).
            tp *= cca * fres *
                  geometrySmithG1GGXAnisotropic(next, h.normal, h.tangent, h.bitangent, sp.roughness, sp.anisotropy) /
                  fmaxf(sp.sP, 1e-5f);
        }
    } else {
        next = diffuseDir;
        tp *= diffuseBounceWeight(m, sp, next) / fmaxf(sp.dP, 1e-5f);
    }
    prevPdf = bsdfPDF(sp, next);
    ray.origin = shadowOrigin;
    ray.direction = next;
    bool dead = terminatePathWithRussianRoulette(bounce, tp, state);
    W.ray_o[p] = make_float4(ray.origin.x, ray.origin.y, ray.origin.z, 0.0f);
    W.ray_d[p] = make_float4(ray.direction.x, ray.direction.y, ray.direction.z, 0.0f);
    W.tp[p] = make_float4(tp.x, tp.y, tp.z, prevPdf);
    W.rng[p] = make_uint2(state, flags);
    out.survive = !dead;
    return out;
}

#ifndef DK_SHADE_MIN_BLOCKS
#define DK_SHADE_MIN_BLOCKS 4
#endif
// range 0: the whole queue; 1: the sorted queue before the subsurface bucket;
// 2: from it on.
template <bool kVolumes, bool kSss>
__global__ void __launch_bounds__(128, DK_SHADE_MIN_BLOCKS) k_shade(DevScene S, Wave W, uint32_t bounce, uint32_t sel,
                                                                  uint32_t sorted, uint32_t range) {
    const uint32_t* q = sorted ? W.qsorted : W.q[sel];
    const uint32_t n = W.counts[sel];
    const uint32_t begin = range == 2u ? W.counts[7] : 0u, end = range == 1u ? W.counts[7] : n;
    if (globalId() == 0) W.counts[4] = 0u;  // extend cursor of the next bounce
    for (uint32_t i = begin + globalId(); i < end; i += gridStride()) {
        uint32_t p = q[i];
        ShadeOut o = shadePath<kVolumes, kSss>(S, W, p, i, bounce);
        bool keep = o.survive && bounce + 1u < o.maxBounces;
        W.live[p] = keep ? 1u : 0u;  // the next queue is built from these flags in path order
        bool sh = o.neeMask != 0u;
        uint32_t sslot = warpAppend(&W.counts[2], sh);
        if (sh) W.qs[sslot] = i;
        for (uint32_t k = 0; k < 3u; ++k) {
            bool has = (o.neeMask >> k) & 1u;
            uint32_t r = warpAppend(&W.counts[3], has);
            if (has) W.qr[r] = (i << 2) | k;
        }
    }
}

// The ordered walk of shadowOccluded (PathTrace.metal:4196-4274) over layers
// collected in (distance, reference slot) order -- the order the reference's
// repeated closest-hit queries meet them: restart 0.001 past each layer,
// transmittance below 0.02 occludes.
__device__ __noinline__ bool walkLayers(const DevScene& S, MatTable mt, float3 o, float3 d, const float* lt,
                                        const uint32_t* ltri, const float* lu, const float* lv, int count, float3& T) {
    float prev = 0.0f;
    bool started = false;
    Ray ray{o, d};
    for (int i = 0; i < count; ++i) {
        float a = lt[i];
        if (started && a <= prev + 0.0015f) continue;  // inside the 0.001 restart gap + 0.0005 epsilon
        float trel = started ? a - (prev + 0.001f) : a;
        HitRec r{a, ltri[i], lu[i], lv[i]};
        Hit h = makeHit(S, ray, r);
        Material sm = materialForHit(S, mt, h);
        prev = a;
        started = true;
        if (sm.baseColor.w <= 0.001f) continue;
        float transmission = materialTransmission(sm);
        bool insideSolid = !h.frontFacing && !materialThinWalled(sm);
        float3 medium = (materialHasVolumeScattering(sm) && insideSolid)
                            ? exp3((-materialVolumeSigmaT(sm)) * trel)
                            : materialTransmissionAbsorption(sm, trel, insideSolid);
        T *= materialTransmissionTint(sm, 0.35f) * medium * transmission;
        if (maxComponent(T) < 0.02f) return true;
    }
    return false;
}

// Inserts a layer into (t, slot) order.
__device__ __forceinline__ void insertLayer(float* lt, uint32_t* ltri, uint32_t* lslot, float* lu, float* lv,
                                            int& count, float t, uint32_t tri, uint32_t slot, float u, float v) {
    int j = count++;
    while (j > 0 && (lt[j - 1] > t || (lt[j - 1] == t && lslot[j - 1] > slot))) {
        lt[j] = lt[j - 1];
        ltri[j] = ltri[j - 1];
        lslot[j] = lslot[j - 1];
        lu[j] = lu[j - 1];
        lv[j] = lv[j - 1];
        --j;
    }
    lt[j] = t;
    ltri[j] = tri;
    lslot[j] = slot;
    lu[j] = u;
    lv[j] = v;
}

// shadowOccluded for scenes with cut-out or transmissive triangles, in one
// traversal: an opaque blocker anywhere in (0.0005, maxDistance) occludes;
// otherwise the non-opaque layers are collected and walked.
// The same collecting traversal over the 8-wide tree.
__device__ __noinline__ bool shadowLayers8(const DevScene& S, MatTable mt, uint32_t opaqueMask, float3 o, float3 d,
                                           float tmax, float3& T) {
    constexpr int kMaxLayers = 8;
    float lt[kMaxLayers];
    uint32_t ltri[kMaxLayers], lslot[kMaxLayers];
    float lu[kMaxLayers], lv[kMaxLayers];
    int count = 0;
    if (S.node_count == 0) return false;
    Trav tr;
    uint2 stack[kTraversalStack];
    travInit(tr, o, d);
    float tm = tmax;
    int r = travSteps(S, tr, stack, tm, 1 << 30, [&](uint32_t i, float&) {
        const float4* q = S.isect + 3 * (size_t)i;
        const float4 a = __ldg(q + 0), b = __ldg(q + 1), c = __ldg(q + 2);
        float t, u, v;
        if (!triTest(S, o, d, a, b, c, t, u, v) || !(t < tmax)) return false;
        if (blocksShadow(__float_as_uint(c.w), opaqueMask)) return true;  // opaque blocker
        if (count == kMaxLayers - 1) return true;                        // an 8th layer: the walk ends occluded
        insertLayer(lt, ltri, lslot, lu, lv, count, t, __float_as_uint(b.w), __float_as_uint(a.w), u, v);
        return false;
    });
    if (r == 2) return true;
    return walkLayers(S, mt, o, d, lt, ltri, lu, lv, count, T);
}

__device__ bool shadowLayers(const DevScene& S, MatTable mt, uint32_t opaqueMask, float3 o, float3 d, float tmax,
                             float3& T) {
    if (S.wide8) return shadowLayers8(S, mt, opaqueMask, o, d, tmax, T);
    constexpr int kMaxLayers = 8;
    float lt[kMaxLayers];
    uint32_t ltri[kMaxLayers], lslot[kMaxLayers];
    float lu[kMaxLayers], lv[kMaxLayers];
    int count = 0;
    float3 inv = rcp3(d);
    int stackNode[kStackSize];
    int sp = 0;
    uint32_t node = 0;
    if (S.node_count == 0) return false;
    for (;;) {
        if ((node & kLeafBit) == 0) {
            Wide w;
            int k = wideVisit(S, node, o, inv, tmax, w);
            if (k > 0) {
                if (k > 3) stackNode[sp++] = (int)w.c3;
                if (k > 2) stackNode[sp++] = (int)w.c2;
                if (k > 1) stackNode[sp++] = (int)w.c1;
                node = w.c0;
                continue;
            }
        } else {
            uint32_t first = (node & ~kLeafBit) >> 3;
            uint32_t cnt = (node & 7u) + 1u;
            for (uint32_t i = first; i < first + cnt; ++i) {
                const float4* q = S.isect + 3 * (size_t)i;
                float4 a = __ldg(q + 0), b = __ldg(q + 1), c = __ldg(q + 2);
                float t, u, v;
                if (!triTest(S, o, d, a, b, c, t, u, v) || !(t < tmax)) continue;
                if (blocksShadow(__float_as_uint(c.w), opaqueMask)) return true;  // opaque blocker
                if (count == kMaxLayers - 1) return true;    // an 8th layer: the walk ends occluded
                insertLayer(lt, ltri, lslot, lu, lv, count, t, __float_as_uint(b.w), __float_as_uint(a.w), u, v);
            }
        }
        if (sp == 0) break;
        node = (uint32_t)stackNode[--sp];
    }
    return walkLayers(S, mt, o, d, lt, ltri, lu, lv, count, T);
}

// The same walk over the (at most kRecLayers) layers the any-hit pass
// recorded: each recorded triangle slot is intersected again with the same
// arithmetic, which reproduces its (t, u, v).
__device__ bool recordedLayers(const DevScene& S, MatTable mt, float3 o, float3 d, const uint2* rec, uint32_t n,
                               float3& T) {
    float lt[kRecLayers];
    uint32_t ltri[kRecLayers], lslot[kRecLayers];
    float lu[kRecLayers], lv[kRecLayers];
    int count = 0;
    for (uint32_t k = 0; k < n && k < kRecLayers; ++k) {
        const float4* q = S.isect + 3 * (size_t)rec[k].y;
        float4 a = __ldg(q + 0), b = __ldg(q + 1), c = __ldg(q + 2);
        float t, u, v;
        if (!triTest(S, o, d, a, b, c, t, u, v)) continue;
        insertLayer(lt, ltri, lslot, lu, lv, count, t, __float_as_uint(b.w), __float_as_uint(a.w), u, v);
    }
    return walkLayers(S, mt, o, d, lt, ltri, lu, lv, count, T);
}

// shadowOccluded (PathTrace.metal:4196-4274) exactly as the reference walks
// it — closest hit per layer, including distance-field hits — for scenes with
// sparse volumes whose layers the single-pass collection does not model.
__device__ bool shadowWalk(const DevScene& S, MatTable mt, float3 o, float3 d, float maxDistance, float3& T) {
    float traveled = 0.0f;
    for (uint32_t step = 0; step < 8u; ++step) {
        sdfCount(S.sdf_counters, kSdfShadowSceneQueries);
        HitRec r = traceSceneCounting(S, o, d);
        if (r.tri == kNoHit || traveled + r.t >= maxDistance) return false;
        Ray ray{o, d};
        Hit h = makeHitAny(S, ray, r);
        Material sm = materialForHit(S, mt, h);
        if (sm.baseColor.w <= 0.001f) {
            traveled += r.t;
            o = h.position + d * 0.001f;
            continue;
        }
        float transmission = materialTransmission(sm);
        if (transmission <= 0.001f) return true;
        bool insideSolid = !h.frontFacing && !materialThinWalled(sm);
        float3 medium = (materialHasVolumeScattering(sm) && insideSolid)
                            ? exp3((-materialVolumeSigmaT(sm)) * r.t)
                            : materialTransmissionAbsorption(sm, r.t, insideSolid);
        T *= materialTransmissionTint(sm, 0.35f) * medium * transmission;
        if (maxComponent(T) < 0.02f) return true;
        traveled += r.t;
        o = h.position + d * 0.001f;
    }
    return true;
}

// Distance-volume closest hit for every ray of the queue, bounded by the
// triangle hit k_extend found (the volume half of intersectScene).
#ifndef DK_VOLUME_MIN_BLOCKS
#define DK_VOLUME_MIN_BLOCKS 4
#endif
// Scenes with one sparse volume (the common case) run it as persistent threads
// with per-lane refill: the volume's grid constants are read once per thread,
// each lane advances its ray `budget` grid cells at a time and takes the next
// ray of the queue when its walk is over.  W.counts[8] is the work cursor
// (zeroed by k_extend).  Measured on the sparse-SDF configuration: budgets of
// 2 / 8 / 32 cells 417 / 570 / 672 Mpaths/s, 64 to 1024 cells 697-698 (a step
// then almost always ends the walk: the per-step ballots cost more than the
// shorter waits for a warp's longest walk save), one ray per thread over the
// general path 493.  Scenes with several volumes, or budget 0
// (DK_VOLUME_REFILL=0), take one ray per thread and walk the volumes in turn.
template <bool kStats>
__global__ void __launch_bounds__(128, DK_VOLUME_MIN_BLOCKS) k_extend_volume(DevScene S, Wave W, uint32_t sel,
                                                                           uint32_t budget) {
    const uint32_t* q = W.q[sel];
    const uint32_t n = W.counts[sel];
    VolumeScene V = volumeScene(S);
    DDAGrid g;
    const bool single = budget && V.volumeCount == 1u && V.gridCount != 0u && V.gridIndexCount != 0u &&
                        V.volumes[0].metadata.w == 1u && ddaGrid(V, 0u, g);
    if (!single) {
        for (uint32_t i = globalId(); i < n; i += gridStride()) {
            uint32_t p = q[i];
            float4 o = W.ray_o[p], d = W.ray_d[p];
            float4 h = W.hit[p];
            VolumeHitRec vh;
            if (kStats ? closestVolumeHitCounted(V, xyz(o), xyz(d), h.x, vh, S.sdf_counters)
                       : closestVolumeHit(V, xyz(o), xyz(d), h.x, vh))
                W.hit[p] = make_float4(vh.t, __uint_as_float(kVolumeHit), __uint_as_float(vh.brick), 0.0f);
        }
        return;
    }
    DDAState st;
    float closestT = 0.0f;
    uint32_t p = kNoWork;
    bool exhausted = false;
    for (;;) {
        uint32_t idx = warpFetch(&W.counts[8], n, p == kNoWork && !exhausted, exhausted);
        if (idx != kNoWork) {
            p = q[idx];
            float4 o = W.ray_o[p], d = W.ray_d[p];
            closestT = W.hit[p].x;
            if (!ddaBegin(g, xyz(o), xyz(d), closestT, st)) p = kNoWork;  // misses the volume's bounds
        }
        if (__all_sync(0xffffffffu, p == kNoWork && exhausted)) break;
        if (p != kNoWork && (kStats ? ddaStepsCounted(V, g, st, (int)budget, S.sdf_counters)
                                    : ddaSteps(V, g, st, (int)budget))) {
            if (st.found && st.out.t < closestT)
                W.hit[p] = make_float4(st.out.t, __uint_as_float(kVolumeHit), __uint_as_float(st.out.brick), 0.0f);
            p = kNoWork;
        }
    }
}

// Shadow rays, persistent threads with per-lane refill: an any-hit query for
// an opaque blocker replaces the slot's unshadowed contribution by its
// shadowed value (contribution / pdf divisor, or 0).  Rays that crossed a
// cut-out or transmissive triangle without meeting an opaque one go to a
// second queue for the layer walk (W.counts[6]).  W.counts[5] is the cursor.
template <bool kWide8>
__global__ void __launch_bounds__(128) k_shadow_rays(DevScene S, Wave W) {
    const uint32_t n = W.counts[3];
    const size_t cap = W.cap;
    // Triangle-only scenes: one scene query per shadow ray (the reference steps through
    // transmissive layers one closest hit at a time; scenes with volumes count the walk's steps).
    if (S.sdf_counters && S.volume_count == 0u && globalId() == 0 && n)
        atomicAdd(S.sdf_counters + kSdfShadowSceneQueries, (unsigned long long)n);
    int stackNode[kWide8 ? 1 : kStackSize];
    uint2 stack8[kWide8 ? kTraversalStack : 1];
    std::conditional_t<kWide8, Any8, AnyState> st;
    uint32_t e = kNoWork;
    bool exhausted = false;
    for (;;) {
        uint32_t idx = warpFetch(&W.counts[5], n, e == kNoWork && !exhausted, exhausted);
        if (idx != kNoWork) {
            e = W.qr[idx];
            size_t slot = (size_t)(e & 3u) * cap + (e >> 2);
            float4 o = W.nee_o[slot], d = W.nee_d[slot];
            anyInit(st, xyz(o), xyz(d), o.w, __ldg(&W.jobs[__float_as_uint(d.w)].opaque_mask),
                    S.volume_count ? nullptr : W.layer_hits + slot * kRecLayers);
        }
        if (__all_sync(0xffffffffu, e == kNoWork && exhausted)) break;
        if (e == kNoWork) continue;
        int r = 1;
        if (S.node_count) {
            if constexpr (kWide8)
                r = anySteps(S, st, stack8, kStepBudget);
            else
                r = anySteps(S, st, stackNode, kStepBudget);
        }
        if (r == 0) continue;
        size_t slot = (size_t)(e & 3u) * cap + (e >> 2);
        if (r == 1 && S.volume_count) st.sawNonOpaque = true;  // distance volumes: the walk decides
        if (r == 2) {
            W.nee_c[slot] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else if (st.sawNonOpaque) {
            W.layer_count[slot] = st.recCount | (st.recOverflow ? 0x80000000u : 0u);
            W.qr2[atomicAdd(&W.counts[6], 1u)] = e;
        } else {
            float4 c = W.nee_c[slot];
            W.nee_c[slot] = make_float4(c.x / c.w, c.y / c.w, c.z / c.w, 0.0f);
        }
        e = kNoWork;
    }
}

// The layer walk for the rays the any-hit pass could not settle: from the
// layers it recorded, or by a collecting traversal when it crossed more.
#ifndef DK_LAYERS_MIN_BLOCKS
#define DK_LAYERS_MIN_BLOCKS 4
#endif
// kVolumes: scenes with sparse volumes walk every shadow ray the reference's
// way (shadowWalk); the others take the recorded layers, or the collecting
// traversal when more were crossed -- two kernels, so that neither carries the
// other's code.
template <bool kVolumes>
__global__ void __launch_bounds__(128, DK_LAYERS_MIN_BLOCKS) k_shadow_layers(DevScene S, Wave W) {
    const uint32_t n = W.counts[6];
    const size_t cap = W.cap;
    for (uint32_t i = globalId(); i < n; i += gridStride()) {
        uint32_t e = W.qr2[i];
        size_t slot = (size_t)(e & 3u) * cap + (e >> 2);
        float4 o = W.nee_o[slot], d = W.nee_d[slot], c = W.nee_c[slot];
        float3 T = f3(1.0f);
        const DevJob& J = W.jobs[__float_as_uint(d.w)];
        const MatTable mt = matTable(J);
        bool occluded;
        if (kVolumes) {
            occluded = shadowWalk(S, mt, xyz(o), xyz(d), o.w, T);
        } else {
            uint32_t lc = W.layer_count[slot];
            occluded = (lc & 0x80000000u)
                           ? shadowLayers(S, mt, __ldg(&J.opaque_mask), xyz(o), xyz(d), o.w, T)
                           : recordedLayers(S, mt, xyz(o), xyz(d), W.layer_hits + slot * kRecLayers, lc, T);
        }
        float3 v = occluded ? f3(0.0f) : xyz(c) * T / c.w;
        W.nee_c[slot] = make_float4(v.x, v.y, v.z, 0.0f);
    }
}

// `radiance += clampSampleContribution(throughput * direct)` with direct the
// sum of the path's shadowed NEE terms in the reference's order (light, env 0,
// env 1; PathTrace.metal:4437-4584, 5396-5421).
__global__ void __launch_bounds__(256) k_resolve(Wave W) {
    const uint32_t n = W.counts[2];
    const size_t cap = W.cap;
    for (uint32_t i = globalId(); i < n; i += gridStride()) {
        uint32_t si = W.qs[i];
        float4 tpw = W.nee_tp[si];
        uint32_t bits = __float_as_uint(tpw.w);
        uint32_t mask = bits & 7u, p = bits >> 3;
        float3 direct = f3(0.0f);
        for (uint32_t k = 0; k < 3u; ++k)
            if (mask & (1u << k)) direct += xyz(W.nee_c[k * cap + si]);
        float4 r = W.rad[p];
        float3 add = clampSampleContribution(xyz(tpw) * direct, __ldg(&W.jobs[jobOf(W, p)].P.clamp));
        W.rad[p] = make_float4(r.x + add.x, r.y + add.y, r.z + add.z, r.w);
    }
}

// tracePrimaryAOV (PathTrace.metal:4093-4159) for the denoiser's unjittered AOV ray.
__global__ void __launch_bounds__(128) k_aov_primary(DevScene S, Wave W) {
    for (uint32_t i = globalId(); i < W.pixel_count; i += gridStride()) {
        const DevJob& J = W.jobs[jobOfPixel(W, i)];
        const DevParams& P = J.P;
        if (P.denoiser == 0u) continue;
        const MatTable mt = matTable(J);
        uint32_t local = i - J.pixel_begin;
        uint32_t px = P.tile_x + local % P.tile_w, py = P.tile_y + local / P.tile_w;
        Ray ray = makeCameraRay(P.cam, P.width, P.height, px, py, 0.5f, 0.5f, 0.0f, 0.0f);
        writeAovMiss(W.aov, i, W.aov_stride);
        for (uint32_t pass = 0; pass < 32u; ++pass) {
            sdfCount(S.sdf_counters, kSdfPrimarySceneQueries);
            HitRec r = traceSceneCounting(S, ray.origin, ray.direction);
            if (r.tri == kNoHit) break;
            Hit h = makeHitAny(S, ray, r);
            Material m = materialForHit(S, mt, h);
            uint32_t nIdx = (uint32_t)m.parameters.w;
            if (nIdx != 0u) h = applyNormalMap(S, h, nIdx, ray.direction);
            uint32_t bIdx = (uint32_t)m.parameters.z;
            if (bIdx != 0u) {
                float4 t = sampleTexture(S, bIdx, h.uv, make_float4(1.0f, 1.0f, 1.0f, 1.0f));
                m.baseColor = make_float4(ex::mul(m.baseColor.x, t.x), ex::mul(m.baseColor.y, t.y),
                                          ex::mul(m.baseColor.z, t.z), ex::mul(m.baseColor.w, t.w));
            }
            if (m.baseColor.w <= 0.001f) {
                ray.origin = ex::add(h.position, ex::mul(ray.direction, 0.001f));
                continue;
            }
            writeAovHit(W.aov, i, W.aov_stride, h, m.baseColor);
            break;
        }
    }
}

// projectToScreen (PathTrace.metal:1662-1697), exact ops.
__device__ bool projectToScreen(const dk_camera& cam, float3 w, uint32_t width, uint32_t height, float2& s) {
    float3 hz = f3(cam.horizontal.x, cam.horizontal.y, cam.horizontal.z);
    float3 vt = f3(cam.vertical.x, cam.vertical.y, cam.vertical.z);
    float3 ll = f3(cam.lower_left.x, cam.lower_left.y, cam.lower_left.z);
    float3 org = f3(cam.origin.x, cam.origin.y, cam.origin.z);
    float3 forward = ex::normalize(ex::cross(vt, hz));
    float3 center = ex::add(ex::add(ll, ex::mul(hz, 0.5f)), ex::mul(vt, 0.5f));
    float3 planePoint;
    if (cam.origin.w > 0.5f) {
        planePoint = ex::sub(w, ex::mul(forward, ex::dot(ex::sub(w, center), forward)));
    } else {
        float3 toPoint = ex::sub(w, org);
        float den = ex::dot(toPoint, forward);
        if (fabsf(den) <= 1e-5f) return false;
        float planeT = ex::div(ex::dot(ex::sub(center, org), forward), den);
        if (planeT <= 0.0f) return false;
        planePoint = ex::add(org, ex::mul(toPoint, planeT));
    }
    float3 rel = ex::sub(planePoint, ll);
    float u = ex::div(ex::dot(rel, hz), fmaxf(ex::dot(hz, hz), 1e-5f));
    float v = ex::div(ex::dot(rel, vt), fmaxf(ex::dot(vt, vt), 1e-5f));
    s = make_float2(ex::mul(u, (float)width), ex::mul(ex::sub(1.0f, v), (float)height));
    return true;
}

// ------------------------------------------- preview and interactive ----
// flatPreviewKernel (PathTrace.metal:4728-4868) and interactiveMaterialKernel
// (:4870-5165), the kernels of RenderQuality.preview and .interactive
// (DenrimRenderer.primaryPipeline, DenrimRenderer.swift:197-214): one camera
// ray through each pixel centre, shaded without path tracing.  Like the
// reference they overwrite the beauty and the AOV planes on every sample
// (the result does not depend on the sample index); the beauty goes into the
// accumulation as one sample.
__device__ __forceinline__ float smoothstepf(float e0, float e1, float x) {  // Metal smoothstep
    float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// sampleInteractiveDiffuseEnvironment (:3805-3823)
__device__ float3 interactiveDiffuseEnv(const DevScene& S, float3 n) {
    float3 up = sampleEnvironment(S, f3(0.0f, 1.0f, 0.0f));
    float3 down = sampleEnvironment(S, f3(0.0f, -1.0f, 0.0f));
    float3 side = (sampleEnvironment(S, f3(1.0f, 0.0f, 0.0f)) + sampleEnvironment(S, f3(-1.0f, 0.0f, 0.0f)) +
                   sampleEnvironment(S, f3(0.0f, 0.0f, 1.0f)) + sampleEnvironment(S, f3(0.0f, 0.0f, -1.0f))) *
                  0.25f;
    float upW = smoothstepf(-0.15f, 0.85f, n.y);
    float downW = smoothstepf(0.15f, -0.85f, n.y);
    float sideW = fmaxf(0.0f, 1.0f - upW - downW);
    return up * upW + down * downW + side * sideW;
}

// interactiveHemisphereDirection (:3825-3831)
__device__ __forceinline__ float3 interactiveHemisphere(float3 d, float3 n) {
    float nd = dot(n, d);
    if (nd < 0.0f) d = d - n * (2.0f * nd);
    return normalize(d);
}

// sampleInteractiveSpecularEnvironment (:3833-3880)
__device__ float3 interactiveSpecularEnv(const DevScene& S, float3 r, float3 n, float roughness) {
    r = interactiveHemisphere(normalize(r), n);
    roughness = clampf(roughness, 0.0f, 1.0f);
    float spread = roughness * roughness;
    float3 helper = fabsf(r.y) < 0.999f ? f3(0.0f, 1.0f, 0.0f) : f3(1.0f, 0.0f, 0.0f);
    float3 t = normalize(cross(helper, r));
    float3 b = cross(r, t);
    float3 cone = sampleEnvironment(S, r) * 0.42f;
    cone += sampleEnvironment(S, interactiveHemisphere(r + t * spread * 0.95f + n * spread * 0.18f, n)) * 0.145f;
    cone += sampleEnvironment(S, interactiveHemisphere(r - t * spread * 0.95f + n * spread * 0.18f, n)) * 0.145f;
    cone += sampleEnvironment(S, interactiveHemisphere(r + b * spread * 0.95f + n * spread * 0.18f, n)) * 0.145f;
    cone += sampleEnvironment(S, interactiveHemisphere(r - b * spread * 0.95f + n * spread * 0.18f, n)) * 0.145f;
    float3 diffuse = interactiveDiffuseEnv(S, n);
    return mix3(cone, diffuse, smoothstepf(0.62f, 0.95f, roughness));
}

// interactiveContactAmbientOcclusion (:4276-4360): four short probes around
// the normal, each nearby occluder weighted by its opacity and proximity.
__device__ float interactiveContactAO(const DevScene& S, MatTable mt, const Hit& h, const Material& m, float3 n) {
    TangentFrame frame = makeTangentFrame(n, h.tangent, h.bitangent);
    constexpr float kRadius = 0.34f;
    const float3 local[4] = {f3(0.000f, 0.000f, 1.000f), f3(0.780f, 0.180f, 0.600f), f3(-0.420f, 0.720f, 0.552f),
                             f3(-0.620f, -0.520f, 0.587f)};
    float occlusion = 0.0f;
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        float3 l = normalize(local[k]);
        float3 dir = normalize(l.x * frame.tangent + l.y * frame.bitangent + l.z * n);
        Ray ray{h.position + n * 0.003f, dir};
        sdfCount(S.sdf_counters, kSdfShadowSceneQueries);
        HitRec r = traceSceneCounting(S, ray.origin, ray.direction);
        if (r.tri == kNoHit || !(r.t < kRadius)) continue;
        Hit oh = makeHitAny(S, ray, r);
        Material om = materialForHit(S, mt, oh);
        float blocker = clampf(om.baseColor.w, 0.0f, 1.0f) * (1.0f - materialTransmission(om) * 0.72f);
        occlusion += blocker * (1.0f - smoothstepf(0.0f, kRadius, r.t));
    }
    float strength = 0.72f + (0.36f - 0.72f) * materialTransmission(m);  // mix(0.72, 0.36, transmission)
    return 1.0f - clampf((occlusion / 4.0f) * strength, 0.0f, 0.72f);
}

template <bool kInteractive>
__global__ void __launch_bounds__(128) k_preview(DevScene S, DevParams P, Accum A, MatTable mt, uint32_t opaqueMask) {
    const uint32_t tileN = P.tile_w * P.tile_h;
    const size_t plane = (size_t)P.width * P.height;
    for (uint32_t i = globalId(); i < tileN; i += gridStride()) {
        const uint32_t px = P.tile_x + i % P.tile_w, py = P.tile_y + i / P.tile_w;
        const size_t pix = (size_t)py * P.width + px;
        Ray ray = makeCameraRay(P.cam, P.width, P.height, px, py, 0.5f, 0.5f, 0.0f, 0.0f);
        sdfCount(S.sdf_counters, kSdfPrimarySceneQueries);
        HitRec rec = traceSceneCounting(S, ray.origin, ray.direction);
        float4 beauty;
        if (rec.tri == kNoHit) {
            float alpha = P.transparent_background ? 0.0f : 1.0f;
            float3 color = mx(f3(P.bg[0], P.bg[1], P.bg[2]), f3(0.0f));
            if (!P.transparent_background && P.shows_env_bg) color = sampleEnvironment(S, ray.direction);
            beauty = make_float4(color.x, color.y, color.z, alpha);
            A.aov[0 * plane + pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            A.aov[1 * plane + pix] = make_float4(0.5f, 0.5f, 0.5f, 0.0f);
            for (int k = 2; k < 6; ++k) A.aov[k * plane + pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else {
            Hit h = makeHitAny(S, ray, rec);
            Material m = materialForHit(S, mt, h);
            uint32_t nIdx = (uint32_t)m.parameters.w;
            if (nIdx != 0u) h = applyNormalMap(S, h, nIdx, ray.direction);
            uint32_t bIdx = (uint32_t)m.parameters.z;
            if (bIdx != 0u) {  // applyBaseColorTexture
                float4 t = sampleTexture(S, bIdx, h.uv, make_float4(1.0f, 1.0f, 1.0f, 1.0f));
                m.baseColor = make_float4(ex::mul(m.baseColor.x, t.x), ex::mul(m.baseColor.y, t.y),
                                          ex::mul(m.baseColor.z, t.z), ex::mul(m.baseColor.w, t.w));
            }
            const float3 n = ex::normalize(h.normal);
            const float3 view = ex::normalize(-ray.direction);
            float3 color;
            float4 albedo;
            if (!kInteractive) {  // :4824-4834
                const float3 key = ex::normalize(f3(0.35f, 0.72f, 0.58f));
                float lambert = fmaxf(ex::dot(n, key), 0.0f);
                float facing = fmaxf(ex::dot(n, view), 0.0f);
                float rim = ex::mul(powf(ex::sub(1.0f, facing), 2.0f), 0.08f);
                float shade = ex::add(ex::add(0.32f, ex::mul(0.68f, lambert)), rim);
                color = ex::add(ex::mul(mx(xyz(m.baseColor), f3(0.0f)), shade), mx(xyz(m.emission), f3(0.0f)));
                beauty = make_float4(color.x, color.y, color.z,
                                     P.transparent_background ? clampf(m.baseColor.w, 0.0f, 1.0f) : 1.0f);
                albedo = m.baseColor;
            } else {  // :4961-5133
                const float roughness = clampf(m.parameters.x, 0.02f, 1.0f);
                const float metallic = clampf(m.parameters.y, 0.0f, 1.0f);
                const float opacity = clampf(m.baseColor.w, 0.0f, 1.0f);
                const float3 base = mx(xyz(m.baseColor), f3(0.0f));
                color = mx(xyz(m.emission), f3(0.0f));
                ShadePoint sp;
                makeShadePoint(sp, m, n, h.tangent, h.bitangent, view);
                const uint32_t nl = min(S.light_count, 12u);
#pragma unroll 1
                for (uint32_t l = 0; l < nl; ++l) {
                    const dk_light_record& L = S.lights[l];
                    if (L.triangle_index >= S.tri_count || L.material_index >= S.mat_count) continue;
                    const dk_triangle& lt = S.tris[L.triangle_index];
                    float3 emission = mx(xyz(__ldg(reinterpret_cast<const float4*>(S.mats + L.material_index) + 1)),
                                         f3(0.0f));
                    if (maxComponent(emission) <= 0.0f || L.area <= 0.0f) continue;
                    float3 lp = (f3(lt.v0.x, lt.v0.y, lt.v0.z) + f3(lt.v1.x, lt.v1.y, lt.v1.z) +
                                 f3(lt.v2.x, lt.v2.y, lt.v2.z)) / 3.0f;
                    float3 toL = lp - h.position;
                    float d2 = fmaxf(dot(toL, toL), 1e-5f);
                    float dist = sqrtf(d2);
                    float3 ld = toL / dist;
                    float cosS = fmaxf(dot(n, ld), 0.0f);
                    float cosL = fmaxf(dot(f3(L.normal.x, L.normal.y, L.normal.z), -ld), 0.0f);
                    if (cosS <= 0.0f || cosL <= 0.0f) continue;
                    float3 T = f3(1.0f);
                    float3 so = h.position + n * 0.001f;
                    if (!S.volume_count) sdfCount(S.sdf_counters, kSdfShadowSceneQueries);
                    bool occluded = S.volume_count ? shadowWalk(S, mt, so, ld, dist - 0.002f, T)
                                                   : shadowLayers(S, mt, opaqueMask, so, ld, dist - 0.002f, T);
                    if (occluded) continue;
                    float3 brdf = evalBRDF(m, sp, ld);
                    float ccGloss = materialClearcoat(m) * powf(1.0f - materialClearcoatRoughness(m), 2.0f);
                    float glossW = clampf(metallic + ccGloss +
                                              (1.0f - metallic) * powf(1.0f - roughness, 4.0f) *
                                                  clampf(m.parameters2.x, 0.0f, 1.0f),
                                          0.0f, 1.0f);
                    float3 f0 = materialF0(m);
                    float3 diffuseOnly = (1.0f - metallic) * base * mx(f3(0.0f), f3(1.0f) - f0) * 0.31830988618f;
                    brdf = mix3(diffuseOnly, brdf, glossW);
                    float G = cosS * cosL * L.area / d2;
                    color += brdf * emission * G * T;
                }
                float3 envDiffuse = interactiveDiffuseEnv(S, n);
                float3 refl = normalize(reflect(-view, n));
                float3 baseRefl = interactiveSpecularEnv(S, refl, n, roughness);
                float ccRough = materialClearcoatRoughness(m);
                float3 ccRefl = interactiveSpecularEnv(S, refl, n, ccRough);
                float nDotV = fmaxf(dot(n, view), 0.0f);
                float3 fresnel = fresnelSchlickThinFilm(nDotV, materialF0(m), m);
                float glossy = powf(1.0f - roughness, 4.0f);
                float metalW = metallic * powf(1.0f - roughness, 2.0f);
                float ccW = materialClearcoat(m) * powf(1.0f - ccRough, 3.0f);
                float dielectricW = (1.0f - metallic) * glossy * clampf(m.parameters2.x, 0.0f, 1.0f);
                float3 roughFresnel = mix3(fresnel, materialF0(m), smoothstepf(0.45f, 0.95f, roughness));
                float3 ccFresnel = fresnelSchlickThinFilm(nDotV, materialClearcoatF0Color(m), m);
                float horizon = 0.58f + 0.42f * clampf(n.y * 0.5f + 0.5f, 0.0f, 1.0f);
                float contact = interactiveContactAO(S, mt, h, m, n);
                float diffuseStrength = 0.58f * (1.0f - metallic) * (horizon * contact);
                float baseReflStrength = metalW * 1.05f + dielectricW * 0.32f;
                color += base * envDiffuse * diffuseStrength;
                color += baseRefl * roughFresnel * baseReflStrength;
                color += ccRefl * ccFresnel * ccW * 0.42f;
                const float3 key = normalize(f3(-0.32f, 0.78f, 0.52f));
                color += base * (1.0f - metallic) * fmaxf(dot(n, key), 0.0f) * 0.16f * contact;
                float subsurface = materialSubsurface(m);
                if (subsurface > 0.0f) {
                    float wrap = powf(1.0f - nDotV, 2.0f);
                    color += clamp3(xyz(m.subsurfaceColor), f3(0.0f), f3(0.999f)) * base * envDiffuse * subsurface *
                             (0.12f + 0.22f * wrap) * contact;
                }
                float transmission = materialTransmission(m);
                if (transmission > 0.0f) {
                    float3 transmitted = sampleEnvironment(S, ray.direction);
                    color = mix3(color, transmitted * materialTransmissionTint(m, 0.65f), transmission * 0.55f);
                    color += baseRefl * fresnel * transmission * 0.35f;
                }
                color = clamp3(color, f3(0.0f), f3(fmaxf(P.clamp, 1.0f)));
                beauty = make_float4(color.x, color.y, color.z, P.transparent_background ? opacity : 1.0f);
                albedo = make_float4(base.x, base.y, base.z, opacity);
            }
            const float3 enc = ex::add(ex::mul(n, 0.5f), f3(0.5f));
            const float mid = (float)(h.materialID + 1u), oid = (float)(h.objectID + 1u);
            A.aov[0 * plane + pix] = make_float4(h.t, h.t, h.t, 1.0f);
            A.aov[1 * plane + pix] = make_float4(enc.x, enc.y, enc.z, 1.0f);
            A.aov[2 * plane + pix] = albedo;
            A.aov[3 * plane + pix] = make_float4(mid, mid, mid, 1.0f);
            A.aov[4 * plane + pix] = make_float4(oid, oid, oid, 1.0f);
            float2 cur, prev;
            if (projectToScreen(P.cam, h.position, P.width, P.height, cur) &&
                projectToScreen(P.prev_cam, h.position, P.width, P.height, prev))
                A.aov[5 * plane + pix] = make_float4(ex::sub(prev.x, cur.x), ex::sub(prev.y, cur.y), 0.0f, 1.0f);
            else
                A.aov[5 * plane + pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        A.sum[pix] = beauty;
        A.comp[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        A.resolved[pix] = D4{0.0, 0.0, 0.0, 0.0};
        A.count[pix] = 1u;
    }
}

// Kahan-compensated accumulation of every path of the batch into its pixel,
// in sample order, plus the AOV block (PathTrace.metal:5559-5585) from the
// batch's last sample.  After every 4096th sample of a pixel the FP32 sum is
// folded into an FP64 resolve buffer, so the result does not depend on how the
// samples were split into batches.
__global__ void __launch_bounds__(256) k_finalize(Wave W) {
    for (uint32_t i = globalId(); i < W.pixel_count; i += gridStride()) {
        const DevJob& J = W.jobs[jobOfPixel(W, i)];
        const DevParams& P = J.P;
        const Accum A = J.A;
        const uint32_t tileN = P.tile_w * P.tile_h;
        uint32_t local = i - J.pixel_begin;
        const float4* rad = W.rad + J.path_begin;
        uint32_t px = P.tile_x + local % P.tile_w, py = P.tile_y + local / P.tile_w;
        size_t pix = (size_t)py * P.width + px;
        float4 s = A.sum[pix], c = A.comp[pix];
        uint32_t count = A.count[pix];
        for (uint32_t k = 0; k < P.samples_in_batch; ++k) {
            float4 r = rad[(size_t)k * tileN + local];
            float y, t;
            y = r.x - c.x; t = s.x + y; c.x = (t - s.x) - y; s.x = t;
            y = r.y - c.y; t = s.y + y; c.y = (t - s.y) - y; s.y = t;
            y = r.z - c.z; t = s.z + y; c.z = (t - s.z) - y; s.z = t;
            y = r.w - c.w; t = s.w + y; c.w = (t - s.w) - y; s.w = t;
            if (((count + k + 1u) & 4095u) == 0u) {  // a 4096-sample block is complete: fold it in FP64
                D4 R = A.resolved[pix];
                R.x += (double)s.x - (double)c.x;
                R.y += (double)s.y - (double)c.y;
                R.z += (double)s.z - (double)c.z;
                R.w += (double)s.w - (double)c.w;
                A.resolved[pix] = R;
                s = make_float4(0, 0, 0, 0);
                c = make_float4(0, 0, 0, 0);
            }
        }
        uint32_t newCount = count + P.samples_in_batch;
        A.sum[pix] = s;
        A.comp[pix] = c;
        A.count[pix] = newCount;
        const size_t st = W.aov_stride;
        float4 a0 = W.aov[i], a1 = W.aov[st + i], a2 = W.aov[2 * st + i], a3 = W.aov[3 * st + i];
        size_t plane = (size_t)P.width * P.height;
        if (__float_as_uint(a0.w) != 0u) {
            float t = a0.x;
            float3 n = f3(a1.x, a1.y, a1.z);
            float3 enc = ex::add(ex::mul(n, 0.5f), f3(0.5f));
            float mid = (float)(__float_as_uint(a0.y) + 1u), oid = (float)(__float_as_uint(a0.z) + 1u);
            A.aov[0 * plane + pix] = make_float4(t, t, t, 1.0f);
            A.aov[1 * plane + pix] = make_float4(enc.x, enc.y, enc.z, 1.0f);
            A.aov[2 * plane + pix] = a2;
            A.aov[3 * plane + pix] = make_float4(mid, mid, mid, 1.0f);
            A.aov[4 * plane + pix] = make_float4(oid, oid, oid, 1.0f);
            float2 cur, prev;
            float3 pos = f3(a3.x, a3.y, a3.z);
            if (projectToScreen(P.cam, pos, P.width, P.height, cur) &&
                projectToScreen(P.prev_cam, pos, P.width, P.height, prev)) {
                A.aov[5 * plane + pix] = make_float4(ex::sub(prev.x, cur.x), ex::sub(prev.y, cur.y), 0.0f, 1.0f);
            } else {
                A.aov[5 * plane + pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
        } else {
            A.aov[0 * plane + pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            A.aov[1 * plane + pix] = make_float4(0.5f, 0.5f, 0.5f, 0.0f);
            A.aov[2 * plane + pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            A.aov[3 * plane + pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            A.aov[4 * plane + pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            A.aov[5 * plane + pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
}

// Beauty resolve for readback: (FP64 resolve + FP32 Kahan sum) / samples.
__global__ void k_resolve_beauty(Accum A, uint32_t pixels, float4* out) {
    for (uint32_t i = globalId(); i < pixels; i += gridStride()) {
        uint32_t n = A.count[i];
        if (n == 0u) {
            out[i] = make_float4(0, 0, 0, 0);
            continue;
        }
        D4 R = A.resolved[i];
        float4 s = A.sum[i], c = A.comp[i];
        double inv = 1.0 / (double)n;
        out[i] = make_float4((float)((R.x + ((double)s.x - (double)c.x)) * inv), (float)((R.y + ((double)s.y - (double)c.y)) * inv),
                             (float)((R.z + ((double)s.z - (double)c.z)) * inv), (float)((R.w + ((double)s.w - (double)c.w)) * inv));
    }
}

// ------------------------------------------ environment importance table --
// environmentSamples (Acceleration/LightingGPUEncoding.swift:66-119) with an
// FP64 weight and prefix sum; stored as FP32 {cdf, pdfSolidAngle}.
__global__ void k_env_weights(const float4* px, uint32_t w, uint32_t h, float intensity, float maxR, double* weights) {
    uint32_t n = w * h;
    double dTheta = 3.141592653589793 / (double)h, dPhi = 2.0 * 3.141592653589793 / (double)w;
    for (uint32_t i = globalId(); i < n; i += gridStride()) {
        uint32_t y = i / w;
        double theta = ((double)y + 0.5) * dTheta;
        double solid = fmax(sin(theta) * dTheta * dPhi, 1e-8);
        float4 t = px[i];
        double r = (double)t.x * intensity, g = (double)t.y * intensity, b = (double)t.z * intensity;
        if (maxR > 0.0f) {
            r = fmin(r, (double)maxR);
            g = fmin(g, (double)maxR);
            b = fmin(b, (double)maxR);
        }
        double lum = r * 0.2126 + g * 0.7152 + b * 0.0722;
        weights[i] = fmax(lum, 0.0) * solid;
    }
}

// Block-local inclusive scan (FP64) of 1024 elements per block; block totals out.
__global__ void __launch_bounds__(1024) k_scan_block(double* data, uint32_t n, double* blockSums) {
    __shared__ double warpSums[32];
    uint32_t i = blockIdx.x * 1024u + threadIdx.x;
    double v = i < n ? data[i] : 0.0;
    for (int o = 1; o < 32; o <<= 1) {
        double u = __shfl_up_sync(0xffffffffu, v, o);
        if ((int)laneId() >= o) v += u;
    }
    if (laneId() == 31u) warpSums[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32u) {
        double ws = warpSums[threadIdx.x];
        for (int o = 1; o < 32; o <<= 1) {
            double u = __shfl_up_sync(0xffffffffu, ws, o);
            if ((int)threadIdx.x >= o) ws += u;
        }
        warpSums[threadIdx.x] = ws;
    }
    __syncthreads();
    if ((threadIdx.x >> 5) > 0u) v += warpSums[(threadIdx.x >> 5) - 1u];
    if (i < n) data[i] = v;
    if (threadIdx.x == 1023u) blockSums[blockIdx.x] = v;
}

// Sequential scan of the (few thousand) block totals, then the finished table.
__global__ void k_scan_totals(double* blockSums, uint32_t nb) {
    if (globalId() != 0) return;
    double acc = 0.0;
    for (uint32_t b = 0; b < nb; ++b) {
        double t = blockSums[b];
        blockSums[b] = acc;
        acc += t;
    }
    blockSums[nb] = acc;
}

__global__ void k_env_finish(const double* prefix, const double* blockSums, const double* weights, uint32_t w,
                             uint32_t h, uint32_t nb, float2* out) {
    uint32_t n = w * h;
    double total = blockSums[nb];
    double dTheta = 3.141592653589793 / (double)h, dPhi = 2.0 * 3.141592653589793 / (double)w;
    for (uint32_t i = globalId(); i < n; i += gridStride()) {
        double cum = prefix[i] + blockSums[i >> 10];
        uint32_t y = i / w;
        double theta = ((double)y + 0.5) * dTheta;
        double solid = fmax(sin(theta) * dTheta * dPhi, 1e-8);
        double prob = weights[i] / total;
        out[i] = make_float2((float)fmin(cum / total, 1.0), (float)(prob / solid));
    }
}

}  // namespace dk

// =========================================================== launchers =====
namespace dk {

int kernelGrid(int which, int smCount) {
    int perSM = 1;
    switch (which) {
        case 0: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_generate, 256, 0); break;
        case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_extend<false>, 128, 0); break;
        case 2: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_shade<false, false>, 128, 0); break;
        case 3: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_shadow_rays<false>, 128, 0); break;
        case 5: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_extend<true>, 128, 0); break;
        case 6: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_shadow_rays<true>, 128, 0); break;
        case 7: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_extend_volume<false>, 128, 0); break;
        default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_finalize, 256, 0); break;
    }
    return (perSM < 1 ? 1 : perSM) * smCount;
}

cudaError_t launchGenerate(const DevScene& S, const Wave& W, int grid, cudaStream_t st) {
    k_generate<<<grid, 256, 0, st>>>(S, W);
    return cudaGetLastError();
}
cudaError_t launchExtend(const DevScene& S, const Wave& W, uint32_t sel, uint32_t bounce, int grid, int volumeGrid,
                         cudaStream_t st) {
    if (S.wide8)
        k_extend<true><<<grid, 128, 0, st>>>(S, W, sel, bounce);
    else
        k_extend<false><<<grid, 128, 0, st>>>(S, W, sel, bounce);
    if (S.volume_count) {
        // grid cells per refill step (DK_VOLUME_BUDGET, default 256); DK_VOLUME_REFILL=0: one ray per thread
        const char* refill = getenv("DK_VOLUME_REFILL");
        const char* env = getenv("DK_VOLUME_BUDGET");
        uint32_t budget = env ? (uint32_t)strtoul(env, nullptr, 10) : 256u;
        budget = budget < 1u ? 1u : (budget > 1024u ? 1024u : budget);
        if (refill && refill[0] == '0') budget = 0u;
        if (S.sdf_counters)  // the counting instantiation only when the session collects them
            k_extend_volume<true><<<volumeGrid, 128, 0, st>>>(S, W, sel, budget);
        else
            k_extend_volume<false><<<volumeGrid, 128, 0, st>>>(S, W, sel, budget);
    }
    return cudaGetLastError();
}
// The environment rotation's sine and cosine with the device's sincosf, the
// values every environment lookup of the reference computes per call.
__global__ void k_env_rotation(float radians, float* out) {
    float sn, cs;
    sincosf(radians, &sn, &cs);
    out[0] = sn;
    out[1] = cs;
}

cudaError_t envRotation(float radians, float* sinCos, cudaStream_t st) {
    k_env_rotation<<<1, 1, 0, st>>>(radians, sinCos);
    return cudaGetLastError();
}

int g_sortMaterials = -1;  // -1: from DK_SORT_MATERIALS (default on)

// Kernels one bounce launches (extend, shade, shadow, resolve stages).
uint32_t bounceLaunches(const DevScene& S) {
    if (g_sortMaterials < 0) {
        const char* e = getenv("DK_SORT_MATERIALS");
        g_sortMaterials = (e && e[0] == '0') ? 0 : 1;
    }
    uint32_t n = 1u + (S.volume_count ? 1u : 0u);                  // extend
    n += 1u + (g_sortMaterials ? (S.volume_count || S.wide8 ? 3u : 4u) : 0u) + 3u;  // sort, shade, survivor queue
    n += 1u + ((!S.all_shadow_opaque || S.volume_count) ? 1u : 0u);  // shadow
    return n + 1u;                                                   // resolve
}

cudaError_t launchShade(const DevScene& S, const Wave& W, uint32_t bounce, uint32_t sel, int grid, cudaStream_t st) {
    if (g_sortMaterials < 0) {
        const char* e = getenv("DK_SORT_MATERIALS");
        g_sortMaterials = (e && e[0] == '0') ? 0 : 1;
    }
    uint32_t sorted = (uint32_t)g_sortMaterials;
    if (sorted) {
        k_sort_count<<<grid, 256, 0, st>>>(S, W, sel);
        k_sort_scan<<<1, kSortBins, 0, st>>>(W);
        k_sort_scatter<<<(W.cap + 256u * kSortItems - 1u) / (256u * kSortItems), 256, 0, st>>>(W, sel);
    }
    // The general shading kernel (volume hits, random walks through
    // traceScene) also serves the 8-wide tree, keeping the layout switch out
    // of the triangle-only kernel.
    if (S.volume_count || S.wide8) {
        k_shade<true, true><<<grid, 128, 0, st>>>(S, W, bounce, sel, sorted, 0u);
    } else if (sorted) {
        // materials without a subsurface weight, then those with one
        k_shade<false, false><<<grid, 128, 0, st>>>(S, W, bounce, sel, sorted, 1u);
        k_shade<false, true><<<grid, 128, 0, st>>>(S, W, bounce, sel, sorted, 2u);
    } else {
        k_shade<false, true><<<grid, 128, 0, st>>>(S, W, bounce, sel, sorted, 0u);
    }
    // The survivors, in path order, are the next bounce's queue.
    const uint32_t blocks = (W.path_count + kLiveBlock - 1u) / kLiveBlock;
    if (blocks) {
        k_live_count<<<blocks, 256, 0, st>>>(W);
        k_live_scan<<<1, 256, 0, st>>>(W, sel, blocks);
        k_live_scatter<<<blocks, 256, 0, st>>>(W, sel);
    } else {
        k_live_scan<<<1, 256, 0, st>>>(W, sel, 0u);
    }
    return cudaGetLastError();
}
cudaError_t launchShadow(const DevScene& S, const Wave& W, int grid, cudaStream_t st) {
    if (S.wide8)
        k_shadow_rays<true><<<grid, 128, 0, st>>>(S, W);
    else
        k_shadow_rays<false><<<grid, 128, 0, st>>>(S, W);
    if (S.volume_count)
        k_shadow_layers<true><<<grid, 128, 0, st>>>(S, W);
    else if (!S.all_shadow_opaque)
        k_shadow_layers<false><<<grid, 128, 0, st>>>(S, W);
    return cudaGetLastError();
}
cudaError_t launchResolve(const Wave& W, int grid, cudaStream_t st) {
    k_resolve<<<grid, 256, 0, st>>>(W);
    return cudaGetLastError();
}
cudaError_t launchAovPrimary(const DevScene& S, const Wave& W, int grid, cudaStream_t st) {
    k_aov_primary<<<grid, 128, 0, st>>>(S, W);
    return cudaGetLastError();
}
cudaError_t launchPreview(const DevScene& S, const DevParams& P, const Accum& A, uint32_t matCount,
                          uint32_t opaqueMask, bool interactive, int grid, cudaStream_t st) {
    const MatTable mt{0u, matCount};
    if (interactive)
        k_preview<true><<<grid, 128, 0, st>>>(S, P, A, mt, opaqueMask);
    else
        k_preview<false><<<grid, 128, 0, st>>>(S, P, A, mt, opaqueMask);
    return cudaGetLastError();
}
cudaError_t launchFinalize(const Wave& W, int grid, cudaStream_t st) {
    k_finalize<<<grid, 256, 0, st>>>(W);
    return cudaGetLastError();
}
cudaError_t launchResolveBeauty(const Accum& A, uint32_t pixels, float4* out, int grid, cudaStream_t st) {
    k_resolve_beauty<<<grid, 256, 0, st>>>(A, pixels, out);
    return cudaGetLastError();
}
cudaError_t buildEnvironmentTable(const float4* dPixels, uint32_t w, uint32_t h, float intensity, float maxR,
                                  double* dWeights, double* dPrefix, double* dBlockSums, float2* dOut, int grid,
                                  cudaStream_t st, double* hostTotal) {
    uint32_t n = w * h;
    uint32_t nb = (n + 1023u) / 1024u;
    k_env_weights<<<grid, 256, 0, st>>>(dPixels, w, h, intensity, maxR, dWeights);
    cudaError_t e = cudaMemcpyAsync(dPrefix, dWeights, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return e;
    k_scan_block<<<nb, 1024, 0, st>>>(dPrefix, n, dBlockSums);
    k_scan_totals<<<1, 32, 0, st>>>(dBlockSums, nb);
    e = cudaMemcpyAsync(hostTotal, dBlockSums + nb, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return e;
    if (!(*hostTotal > 0.0)) return cudaSuccess;
    k_env_finish<<<grid, 256, 0, st>>>(dPrefix, dBlockSums, dWeights, w, h, nb, dOut);
    return cudaGetLastError();
}

}  // namespace dk
