// Sparse distance-volume bricks on sm_103a: the brick-grid DDA with macro-cell
// skipping, the per-brick march / bisection / Catmull-Rom polish and the
// gradient normal of the reference's closestVolumeHit for sparse volumes
// (Sources/DenrimRendererKit/Resources/Shaders/PathTrace.metal:1865-1881,
// 2057-2469, 2608-2807, 2862-3263).  All arithmetic uses explicitly rounded
// IEEE operations so that hits on the distance field — and the depth, normal
// and ID AOVs derived from them — match the reference arithmetic bit for bit.
// The march reads the distances from a distance-only copy of the packed
// samples (the same values as the reference's 16-byte records): FP32, or FP16
// (2 bytes per sample) when every distance is a half-precision value.
#pragma once
#include <cuda_fp16.h>

#include "dk_device.cuh"

namespace dk {

constexpr uint32_t kVolumeHit = 0xfffffffeu;

// matrixFromColumns(c0..c3) * float4(v, w).
__device__ __forceinline__ float3 mulColumns(const dk_float4* c, float3 v, float w) {
    float3 r;
    r.x = ex::add(ex::add(ex::add(ex::mul(c[0].x, v.x), ex::mul(c[1].x, v.y)), ex::mul(c[2].x, v.z)), ex::mul(c[3].x, w));
    r.y = ex::add(ex::add(ex::add(ex::mul(c[0].y, v.x), ex::mul(c[1].y, v.y)), ex::mul(c[2].y, v.z)), ex::mul(c[3].y, w));
    r.z = ex::add(ex::add(ex::add(ex::mul(c[0].z, v.x), ex::mul(c[1].z, v.y)), ex::mul(c[2].z, v.z)), ex::mul(c[3].z, w));
    return r;
}

__device__ __forceinline__ float exMix(float a, float b, float t) { return ex::add(a, ex::mul(ex::sub(b, a), t)); }
__device__ __forceinline__ float3 exDiv(float3 a, float3 b) { return f3(ex::div(a.x, b.x), ex::div(a.y, b.y), ex::div(a.z, b.z)); }
__device__ __forceinline__ float3 ld3f(const dk_float4& v) { return f3(v.x, v.y, v.z); }
__device__ __forceinline__ float exLength(float3 v) { return __fsqrt_rn(ex::dot(v, v)); }

// intersectAABB (:1865-1881).
__device__ __forceinline__ bool intersectAABB(float3 o, float3 d, float3 bmin, float3 bmax, float closestT, float& tNear,
                                              float& tFar) {
    float3 inv = rcp3(d);
    float tx0 = ex::mul(ex::sub(bmin.x, o.x), inv.x), tx1 = ex::mul(ex::sub(bmax.x, o.x), inv.x);
    float ty0 = ex::mul(ex::sub(bmin.y, o.y), inv.y), ty1 = ex::mul(ex::sub(bmax.y, o.y), inv.y);
    float tz0 = ex::mul(ex::sub(bmin.z, o.z), inv.z), tz1 = ex::mul(ex::sub(bmax.z, o.z), inv.z);
    tNear = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0005f));
    tFar = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), closestT));
    return tNear <= tFar;
}

struct BrickCtx {
    uint32_t dims[3];
    uint32_t sampleOffset, strideY, strideZ;
    float3 sampleMin, sampleMax, sampleExtent;
    bool valid;
};

// makeVolumeBrickSampleContext (:2075-2095).
__device__ __forceinline__ BrickCtx makeBrickCtx(const dk_volume_brick_descriptor& b, uint64_t brickSampleCount) {
    BrickCtx c;
    uint4 ds = __ldg(reinterpret_cast<const uint4*>(&b.dimensions_and_sample_offset));
    c.dims[0] = ds.x;
    c.dims[1] = ds.y;
    c.dims[2] = ds.z;
    c.sampleOffset = ds.w;
    uint32_t count = ds.x * ds.y * ds.z;
    c.strideY = ds.x;
    c.strideZ = ds.x * ds.y;
    c.sampleMin = ld3f(b.sample_bounds_min);
    c.sampleMax = ld3f(b.sample_bounds_max);
    c.sampleExtent = mx(ex::sub(c.sampleMax, c.sampleMin), f3(1e-6f));
    bool rangeValid = c.sampleOffset < brickSampleCount && count <= brickSampleCount - c.sampleOffset;
    c.valid = ds.x >= 2u && ds.y >= 2u && ds.z >= 2u && rangeValid;
    return c;
}

struct GridPos {
    uint32_t base[3], next[3];
    float frac[3];
};

__device__ __forceinline__ GridPos gridPos(const BrickCtx& c, float3 p) {
    float3 uvw = clamp3(exDiv(ex::sub(p, c.sampleMin), c.sampleExtent), f3(0.0f), f3(1.0f));
    float g[3] = {ex::mul(uvw.x, (float)(c.dims[0] - 1u)), ex::mul(uvw.y, (float)(c.dims[1] - 1u)),
                  ex::mul(uvw.z, (float)(c.dims[2] - 1u))};
    GridPos r;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        r.base[a] = (uint32_t)floorf(g[a]);
        r.next[a] = min(r.base[a] + 1u, c.dims[a] - 1u);
        r.frac[a] = ex::sub(g[a], (float)r.base[a]);
    }
    return r;
}

// The march's distance samples: FP32, or FP16 when every stored distance of
// the scene is exactly a half-precision value (a build with FP16 distances);
// both give the same float.
struct DistSrc {
    const float* f32;
    const uint16_t* f16;
};

// The two sample formats as template arguments of the march, so that the
// format is decided once per brick and not per sample.
struct DistF32 {
    const float* p;
    __device__ __forceinline__ float at(size_t k) const { return __ldg(p + k); }
};
struct DistF16 {
    const uint16_t* p;
    __device__ __forceinline__ float at(size_t k) const { return __half2float(__ushort_as_half(__ldg(p + k))); }
};

template <class D>
__device__ __forceinline__ float sampleD(const D& dist, const BrickCtx& c, uint32_t x, uint32_t y, uint32_t z) {
    return dist.at(c.sampleOffset + x + y * c.strideY + z * c.strideZ);
}

// sampleVolumeBrickDistancePrepared (:2097-2125).
template <class D>
__device__ float brickDistance(const D& dist, const BrickCtx& c, float3 p) {
    if (!c.valid) return INFINITY;
    GridPos g = gridPos(c, p);
    const uint32_t *b = g.base, *n = g.next;
    float c00 = exMix(sampleD(dist, c, b[0], b[1], b[2]), sampleD(dist, c, n[0], b[1], b[2]), g.frac[0]);
    float c10 = exMix(sampleD(dist, c, b[0], n[1], b[2]), sampleD(dist, c, n[0], n[1], b[2]), g.frac[0]);
    float c01 = exMix(sampleD(dist, c, b[0], b[1], n[2]), sampleD(dist, c, n[0], b[1], n[2]), g.frac[0]);
    float c11 = exMix(sampleD(dist, c, b[0], n[1], n[2]), sampleD(dist, c, n[0], n[1], n[2]), g.frac[0]);
    float c0 = exMix(c00, c10, g.frac[1]);
    float c1 = exMix(c01, c11, g.frac[1]);
    return exMix(c0, c1, g.frac[2]);
}

struct DistGrad {
    float distance;
    float3 gradient;
};

// sampleVolumeBrickDistanceGradientPrepared (:2164-2218).
template <class D>
__device__ DistGrad brickDistGrad(const D& dist, const BrickCtx& c, float3 p) {
    DistGrad r;
    r.distance = INFINITY;
    r.gradient = f3(0.0f);
    if (!c.valid) return r;
    GridPos g = gridPos(c, p);
    const uint32_t *b = g.base, *n = g.next;
    const float* f = g.frac;
    float d000 = sampleD(dist, c, b[0], b[1], b[2]), d100 = sampleD(dist, c, n[0], b[1], b[2]);
    float d010 = sampleD(dist, c, b[0], n[1], b[2]), d110 = sampleD(dist, c, n[0], n[1], b[2]);
    float d001 = sampleD(dist, c, b[0], b[1], n[2]), d101 = sampleD(dist, c, n[0], b[1], n[2]);
    float d011 = sampleD(dist, c, b[0], n[1], n[2]), d111 = sampleD(dist, c, n[0], n[1], n[2]);
    float c00 = exMix(d000, d100, f[0]), c10 = exMix(d010, d110, f[0]);
    float c01 = exMix(d001, d101, f[0]), c11 = exMix(d011, d111, f[0]);
    float c0 = exMix(c00, c10, f[1]), c1 = exMix(c01, c11, f[1]);
    r.distance = exMix(c0, c1, f[2]);
    float dx = exMix(exMix(ex::sub(d100, d000), ex::sub(d110, d010), f[1]), exMix(ex::sub(d101, d001), ex::sub(d111, d011), f[1]), f[2]);
    float dy = exMix(exMix(ex::sub(d010, d000), ex::sub(d110, d100), f[0]), exMix(ex::sub(d011, d001), ex::sub(d111, d101), f[0]), f[2]);
    float dz = ex::sub(c1, c0);
    float3 g2l = exDiv(f3((float)(c.dims[0] - 1u), (float)(c.dims[1] - 1u), (float)(c.dims[2] - 1u)), c.sampleExtent);
    r.gradient = f3(ex::mul(dx, g2l.x), ex::mul(dy, g2l.y), ex::mul(dz, g2l.z));
    return r;
}

// cubicCatmullRom / cubicCatmullRomDerivative (:2135-2153).
__device__ __forceinline__ float catmull(float p0, float p1, float p2, float p3, float t) {
    float t2 = ex::mul(t, t), t3 = ex::mul(t2, t);
    float a = ex::mul(2.0f, p1);
    float b = ex::mul(ex::add(-p0, p2), t);
    float c = ex::mul(ex::sub(ex::add(ex::sub(ex::mul(2.0f, p0), ex::mul(5.0f, p1)), ex::mul(4.0f, p2)), p3), t2);
    float d = ex::mul(ex::add(ex::sub(ex::add(-p0, ex::mul(3.0f, p1)), ex::mul(3.0f, p2)), p3), t3);
    return ex::mul(0.5f, ex::add(ex::add(ex::add(a, b), c), d));
}
__device__ __forceinline__ float catmullD(float p0, float p1, float p2, float p3, float t) {
    float t2 = ex::mul(t, t);
    float a = ex::add(-p0, p2);
    float b = ex::mul(ex::mul(2.0f, ex::sub(ex::add(ex::sub(ex::mul(2.0f, p0), ex::mul(5.0f, p1)), ex::mul(4.0f, p2)), p3)), t);
    float c = ex::mul(ex::mul(3.0f, ex::add(ex::sub(ex::add(-p0, ex::mul(3.0f, p1)), ex::mul(3.0f, p2)), p3)), t2);
    return ex::mul(0.5f, ex::add(ex::add(a, b), c));
}

// sampleVolumeBrickDistanceGradientCubicPrepared (:2256-2307).
template <class D>
__device__ __noinline__ DistGrad brickDistGradCubic(const D& dist, const BrickCtx& c, float3 p) {
    if (!c.valid) {
        DistGrad r;
        r.distance = INFINITY;
        r.gradient = f3(0.0f);
        return r;
    }
    float3 uvw = clamp3(exDiv(ex::sub(p, c.sampleMin), c.sampleExtent), f3(0.0f), f3(1.0f));
    float g[3] = {ex::mul(uvw.x, (float)(c.dims[0] - 1u)), ex::mul(uvw.y, (float)(c.dims[1] - 1u)),
                  ex::mul(uvw.z, (float)(c.dims[2] - 1u))};
    uint32_t base[3] = {(uint32_t)floorf(g[0]), (uint32_t)floorf(g[1]), (uint32_t)floorf(g[2])};
    if (base[0] < 1u || base[1] < 1u || base[2] < 1u || base[0] + 2u >= c.dims[0] || base[1] + 2u >= c.dims[1] ||
        base[2] + 2u >= c.dims[2])
        return brickDistGrad(dist, c, p);
    float f[3] = {ex::sub(g[0], (float)base[0]), ex::sub(g[1], (float)base[1]), ex::sub(g[2], (float)base[2])};
    float xr[4][4], dxr[4][4];
#pragma unroll
    for (uint32_t z = 0; z < 4u; ++z)
#pragma unroll
        for (uint32_t y = 0; y < 4u; ++y) {
            uint32_t cy = base[1] + y - 1u, cz = base[2] + z - 1u;
            float p0 = sampleD(dist, c, base[0] - 1u, cy, cz);
            float p1 = sampleD(dist, c, base[0], cy, cz);
            float p2 = sampleD(dist, c, base[0] + 1u, cy, cz);
            float p3 = sampleD(dist, c, base[0] + 2u, cy, cz);
            xr[y][z] = catmull(p0, p1, p2, p3, f[0]);
            dxr[y][z] = catmullD(p0, p1, p2, p3, f[0]);
        }
    float yr[4], dyr[4], dxyr[4];
#pragma unroll
    for (uint32_t z = 0; z < 4u; ++z) {
        yr[z] = catmull(xr[0][z], xr[1][z], xr[2][z], xr[3][z], f[1]);
        dyr[z] = catmullD(xr[0][z], xr[1][z], xr[2][z], xr[3][z], f[1]);
        dxyr[z] = catmull(dxr[0][z], dxr[1][z], dxr[2][z], dxr[3][z], f[1]);
    }
    DistGrad r;
    r.distance = catmull(yr[0], yr[1], yr[2], yr[3], f[2]);
    float dx = catmull(dxyr[0], dxyr[1], dxyr[2], dxyr[3], f[2]);
    float dy = catmull(dyr[0], dyr[1], dyr[2], dyr[3], f[2]);
    float dz = catmullD(yr[0], yr[1], yr[2], yr[3], f[2]);
    float3 g2l = exDiv(f3((float)(c.dims[0] - 1u), (float)(c.dims[1] - 1u), (float)(c.dims[2] - 1u)), c.sampleExtent);
    r.gradient = f3(ex::mul(dx, g2l.x), ex::mul(dy, g2l.y), ex::mul(dz, g2l.z));
    return r;
}

// sampleVolumeBrickCentralGradientPrepared (:2220-2254).
template <class D>
__device__ float3 brickCentralGradient(const D& dist, const BrickCtx& c, float3 p, float3 s) {
    float3 x0 = p, x1 = p, y0 = p, y1 = p, z0 = p, z1 = p;
    x0.x = fmaxf(ex::sub(p.x, s.x), c.sampleMin.x);
    x1.x = fminf(ex::add(p.x, s.x), c.sampleMax.x);
    float dx = ex::div(ex::sub(brickDistance(dist, c, x1), brickDistance(dist, c, x0)), fmaxf(ex::sub(x1.x, x0.x), 1e-6f));
    y0.y = fmaxf(ex::sub(p.y, s.y), c.sampleMin.y);
    y1.y = fminf(ex::add(p.y, s.y), c.sampleMax.y);
    float dy = ex::div(ex::sub(brickDistance(dist, c, y1), brickDistance(dist, c, y0)), fmaxf(ex::sub(y1.y, y0.y), 1e-6f));
    z0.z = fmaxf(ex::sub(p.z, s.z), c.sampleMin.z);
    z1.z = fminf(ex::add(p.z, s.z), c.sampleMax.z);
    float dz = ex::div(ex::sub(brickDistance(dist, c, z1), brickDistance(dist, c, z0)), fmaxf(ex::sub(z1.z, z0.z), 1e-6f));
    return f3(dx, dy, dz);
}

struct VolumeScene {
    const dk_volume_descriptor* volumes;
    const dk_volume_brick_descriptor* bricks;
    const dk_volume_brick_sample* samples;
    DistSrc dist;
    const dk_volume_brick_grid* grids;
    const uint32_t* gridIndices;
    uint64_t sampleCount, gridIndexCount;
    uint32_t volumeCount, brickCount, gridCount;
};

// The reference's SDF traversal counter slots (PathTrace.metal:191-203).
enum : uint32_t {
    kSdfDenseVolumeTests = 0, kSdfDenseMarchSteps = 1, kSdfGridCellsVisited = 2, kSdfGridMacroSkips = 3,
    kSdfBrickTests = 4, kSdfBrickInvalid = 5, kSdfBrickRangeCulls = 6, kSdfBrickMarches = 7,
    kSdfBrickMarchSteps = 8, kSdfBrickHits = 9, kSdfPrimarySceneQueries = 10, kSdfBounceSceneQueries = 11,
    kSdfShadowSceneQueries = 12, kSdfCounterCount = 13
};

// addSDFTraversalCounter (PathTrace.metal:205-214): one event per calling
// lane, aggregated over the lanes that arrive together (one atomic per warp);
// nothing when collection is off (null).
__device__ __forceinline__ void sdfCount(unsigned long long* counters, uint32_t k) {
    if (!counters) return;
    const unsigned m = __activemask();
    if ((threadIdx.x & 31u) == (uint32_t)(__ffs(m) - 1)) atomicAdd(counters + k, (unsigned long long)__popc(m));
}

__device__ __forceinline__ float cellSizeOf(const dk_volume_descriptor& vol) {
    float3 ext = mx(ex::sub(ld3f(vol.local_bounds_max), ld3f(vol.local_bounds_min)), f3(1e-6f));
    float3 den = mx(ex::sub(f3((float)vol.dimensions.x, (float)vol.dimensions.y, (float)vol.dimensions.z), f3(1.0f)), f3(1.0f));
    float3 sp = exDiv(ext, den);
    return fminf(sp.x, fminf(sp.y, sp.z));
}

// volumeBrickNormal (:2420-2469).
template <class D>
__device__ __noinline__ float3 brickNormalT(const D& dist, const dk_volume_descriptor& vol, const BrickCtx& c, float3 p,
                                           bool cubic, bool coarse) {
    if (!c.valid) return f3(0, 1, 0);
    float3 n = cubic ? brickDistGradCubic(dist, c, p).gradient : brickDistGrad(dist, c, p).gradient;
    if (coarse) {
        float3 ext = mx(ex::sub(ld3f(vol.local_bounds_max), ld3f(vol.local_bounds_min)), f3(1e-6f));
        float3 den = mx(ex::sub(f3((float)vol.dimensions.x, (float)vol.dimensions.y, (float)vol.dimensions.z), f3(1.0f)), f3(1.0f));
        float3 spacing = exDiv(ext, den);
        float3 central = brickCentralGradient(dist, c, p, ex::mul(spacing, 1.5f));
        if (ex::dot(central, central) > 1e-10f) {
            float3 a = ex::normalize(n), b = ex::normalize(central);
            n = ex::normalize(f3(exMix(a.x, b.x, 0.35f), exMix(a.y, b.y, 0.35f), exMix(a.z, b.z, 0.35f)));
        }
    }
    if (ex::dot(n, n) <= 1e-10f) n = f3(0, 1, 0);
    return ex::normalize(mulColumns(vol.normal_transform, ex::normalize(n), 0.0f));
}

__device__ __forceinline__ float3 brickNormal(const VolumeScene& V, const dk_volume_descriptor& vol, const BrickCtx& c,
                                              float3 p, bool cubic, bool coarse) {
    if (V.dist.f16) return brickNormalT(DistF16{V.dist.f16}, vol, c, p, cubic, coarse);
    return brickNormalT(DistF32{V.dist.f32}, vol, c, p, cubic, coarse);
}

struct VolumeHitRec {
    float t;
    uint32_t brick;
};

struct VolumeRay {
    float3 lo, ld;
    float upw, cellSize;
};

__device__ __forceinline__ VolumeRay volumeRay(const dk_volume_descriptor& vol, float3 o, float3 d) {
    VolumeRay r;
    r.lo = mulColumns(vol.world_to_local, o, 1.0f);
    r.ld = mulColumns(vol.world_to_local, d, 0.0f);
    r.upw = fmaxf(exLength(r.ld), 1e-6f);
    r.cellSize = cellSizeOf(vol);
    return r;
}

// closestSparseVolumeBrickDDAHit (:2881-3088) in three parts, so that a
// persistent kernel can advance each lane's ray a few cells at a time and
// refill lanes whose ray is done (the operations and their order are those of
// the reference's single loop; sparseDDAHit below runs them back to back).
// The grid of volume `vi` (uniform over a launch):
struct DDAGrid {
    const dk_volume_descriptor* vol;
    uint32_t gd[3], gridOffset, bsz[3];
    uint32_t md[3], macroOffset, msz[3];
    bool hasMacro;
    uint32_t maxSteps;
};
// One ray's walk through it:
struct DDAState {
    VolumeRay vr;
    float bpa[3], va[3], tMax[3], tDelta[3];
    int cell[3], stepDir[3];
    float t, tNear, tFar, closest;
    uint32_t step;
    bool found;
    VolumeHitRec out;
};

// The brick grid of volume `vi`; false when it has none.
__device__ __forceinline__ bool ddaGrid(const VolumeScene& V, uint32_t vi, DDAGrid& g) {
    const dk_volume_brick_grid* grid = nullptr;
    for (uint32_t i = 0; i < V.gridCount; ++i)
        if (V.grids[i].brick_size_and_volume.w == vi) {
            grid = &V.grids[i];
            break;
        }
    if (!grid || !V.gridIndices) return false;
    g.vol = &V.volumes[vi];
    g.gd[0] = grid->dimensions_and_index_offset.x;
    g.gd[1] = grid->dimensions_and_index_offset.y;
    g.gd[2] = grid->dimensions_and_index_offset.z;
    g.gridOffset = grid->dimensions_and_index_offset.w;
    g.bsz[0] = max(grid->brick_size_and_volume.x, 1u);
    g.bsz[1] = max(grid->brick_size_and_volume.y, 1u);
    g.bsz[2] = max(grid->brick_size_and_volume.z, 1u);
    if (g.gd[0] == 0u || g.gd[1] == 0u || g.gd[2] == 0u) return false;
    g.md[0] = grid->macro_dimensions_and_index_offset.x;
    g.md[1] = grid->macro_dimensions_and_index_offset.y;
    g.md[2] = grid->macro_dimensions_and_index_offset.z;
    g.macroOffset = grid->macro_dimensions_and_index_offset.w;
    g.msz[0] = max(grid->macro_size_and_reserved.x, 1u);
    g.msz[1] = max(grid->macro_size_and_reserved.y, 1u);
    g.msz[2] = max(grid->macro_size_and_reserved.z, 1u);
    g.hasMacro = g.md[0] > 0u && g.md[1] > 0u && g.md[2] > 0u && g.macroOffset < V.gridIndexCount;
    g.maxSteps = min(g.gd[0] + g.gd[1] + g.gd[2] + 8u, 1024u);
    return true;
}

// The ray's entry into the volume's bounds and its first cell; false when it
// misses the bounds before closestT (no hit).
__device__ __forceinline__ bool ddaBegin(const DDAGrid& g, float3 o, float3 d, float closestT, DDAState& s) {
    const dk_volume_descriptor& vol = *g.vol;
    if (!intersectAABB(o, d, ld3f(vol.world_bounds_min), ld3f(vol.world_bounds_max), closestT, s.tNear, s.tFar))
        return false;
    s.vr = volumeRay(vol, o, d);
    float3 extent = mx(ex::sub(ld3f(vol.local_bounds_max), ld3f(vol.local_bounds_min)), f3(1e-6f));
    float3 sampleDen = mx(ex::sub(f3((float)vol.dimensions.x, (float)vol.dimensions.y, (float)vol.dimensions.z), f3(1.0f)), f3(1.0f));
    float3 bsf = mx(f3((float)g.bsz[0], (float)g.bsz[1], (float)g.bsz[2]), f3(1.0f));
    s.t = s.tNear;
    float3 lp = ex::add(s.vr.lo, ex::mul(s.vr.ld, s.t));
    float3 sp = exDiv(ex::sub(lp, ld3f(vol.local_bounds_min)), extent);
    sp = f3(ex::mul(sp.x, sampleDen.x), ex::mul(sp.y, sampleDen.y), ex::mul(sp.z, sampleDen.z));
    float3 bp = exDiv(ex::add(sp, f3(0.5f)), bsf);
    s.bpa[0] = bp.x;
    s.bpa[1] = bp.y;
    s.bpa[2] = bp.z;
    float3 vel3 = exDiv(exDiv(s.vr.ld, extent), f3(1.0f));
    vel3 = f3(ex::mul(vel3.x, sampleDen.x), ex::mul(vel3.y, sampleDen.y), ex::mul(vel3.z, sampleDen.z));
    vel3 = exDiv(vel3, bsf);
    s.va[0] = vel3.x;
    s.va[1] = vel3.y;
    s.va[2] = vel3.z;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        s.cell[a] = (int)clampf(floorf(s.bpa[a]), 0.0f, ex::sub((float)g.gd[a], 1.0f));
        s.stepDir[a] = s.va[a] > 0.0f ? 1 : (s.va[a] < 0.0f ? -1 : 0);
        float nb = s.stepDir[a] > 0 ? ex::add((float)s.cell[a], 1.0f) : (float)s.cell[a];
        s.tMax[a] = s.stepDir[a] == 0 ? INFINITY : ex::add(s.t, ex::div(ex::sub(nb, s.bpa[a]), s.va[a]));
        s.tDelta[a] = s.stepDir[a] == 0 ? INFINITY : fabsf(ex::div(1.0f, s.va[a]));
    }
    s.step = 0u;
    s.found = false;
    s.closest = closestT;
    return true;
}

// The walk without counters, then with them (dk_sdf_walk.inc).
#define DK_WALK(name) name
#define DK_WALK_PARAMS
#define DK_WALK_ARGS
#define DK_WALK_COUNT(k)
#define DK_WALK_COUNT_TRUE(k) true
#include "dk_sdf_walk.inc"
#undef DK_WALK
#undef DK_WALK_PARAMS
#undef DK_WALK_ARGS
#undef DK_WALK_COUNT
#undef DK_WALK_COUNT_TRUE
#define DK_WALK(name) name##Counted
#define DK_WALK_PARAMS , unsigned long long* counters
#define DK_WALK_ARGS , counters
#define DK_WALK_COUNT(k) sdfCount(counters, k)
#define DK_WALK_COUNT_TRUE(k) (sdfCount(counters, k), true)
#include "dk_sdf_walk.inc"
#undef DK_WALK
#undef DK_WALK_PARAMS
#undef DK_WALK_ARGS
#undef DK_WALK_COUNT
#undef DK_WALK_COUNT_TRUE

// closestSparseVolumeBrickDDAHit (:2881-3088) for volume `vi`; the Counted
// form counts into `counters`.
__device__ bool sparseDDAHit(const VolumeScene& V, uint32_t vi, float3 o, float3 d, float closestT, VolumeHitRec& out) {
    DDAGrid g;
    if (!ddaGrid(V, vi, g)) return false;
    DDAState s;
    if (!ddaBegin(g, o, d, closestT, s)) return false;
    while (!ddaSteps(V, g, s, 1 << 20)) {
    }
    if (s.found) out = s.out;
    return s.found;
}
__device__ bool sparseDDAHitCounted(const VolumeScene& V, uint32_t vi, float3 o, float3 d, float closestT,
                                    VolumeHitRec& out, unsigned long long* counters) {
    DDAGrid g;
    if (!ddaGrid(V, vi, g)) return false;
    DDAState s;
    if (!ddaBegin(g, o, d, closestT, s)) return false;
    while (!ddaStepsCounted(V, g, s, 1 << 20, counters)) {
    }
    if (s.found) out = s.out;
    return s.found;
}

// closestVolumeHit (:3090-3157), sparse-brick volumes only; the Counted form
// counts into `counters`.
__device__ __noinline__ bool closestVolumeHit(const VolumeScene& V, float3 o, float3 d, float closestT, VolumeHitRec& out) {
    if (V.volumeCount == 0 || V.gridCount == 0 || V.gridIndexCount == 0) return false;
    bool found = false;
    float closest = closestT;
    for (uint32_t i = 0; i < V.volumeCount; ++i) {
        if (V.volumes[i].metadata.w != 1u) continue;
        VolumeHitRec r;
        if (sparseDDAHit(V, i, o, d, closest, r) && r.t < closest) {
            closest = r.t;
            out = r;
            found = true;
        }
    }
    return found;
}
__device__ __noinline__ bool closestVolumeHitCounted(const VolumeScene& V, float3 o, float3 d, float closestT,
                                                    VolumeHitRec& out, unsigned long long* counters) {
    if (V.volumeCount == 0 || V.gridCount == 0 || V.gridIndexCount == 0) return false;
    bool found = false;
    float closest = closestT;
    for (uint32_t i = 0; i < V.volumeCount; ++i) {
        if (V.volumes[i].metadata.w != 1u) continue;
        VolumeHitRec r;
        if (sparseDDAHitCounted(V, i, o, d, closest, r, counters) && r.t < closest) {
            closest = r.t;
            out = r;
            found = true;
        }
    }
    return found;
}
// One call site for the scene query: the counting form when `counters` is set.
__device__ __noinline__ bool closestVolumeHitAny(const VolumeScene& V, float3 o, float3 d, float closestT,
                                                VolumeHitRec& out, unsigned long long* counters) {
    return counters ? closestVolumeHitCounted(V, o, d, closestT, out, counters)
                    : closestVolumeHit(V, o, d, closestT, out);
}

}  // namespace dk
