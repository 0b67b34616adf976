// Scene-compile helper for sparse distance-volume bricks (host side).
//
// Restates, for models made of sphere primitives combined by (smooth) union,
//   * DistanceVolumeBuilder.buildSparse (Scene/SDFModel.swift:255-355) with
//     sampleBrick / samplePosition / sampleField / combine (:357-580): 2-voxel
//     stored overlap, narrow-band brick selection on the stored samples;
//   * LinearTriangleAccelerationBackend.gpuVolumeBricks
//     (Acceleration/SparseVolumeGPUEncoding.swift:9-299): brick descriptors with
//     core / sample bounds and the distance range, packed samples, the brick
//     grid (UInt32.max = empty) and the 4^3 macro-cell occupancy appended to the
//     same index buffer;
//   * appendSparseVolumeDescriptor (Acceleration/VolumeGPUEncoding.swift:184-243)
//     for an identity instance transform.
// Bricks whose stored samples provably lie outside the narrow band are skipped
// without sampling: the polynomial smooth minimum is monotone in both
// arguments, so running the union chain on per-sphere [min, max] distance
// intervals over the brick bounds the field of every sample in it.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/denrim_cuda.h"

namespace dk {
void setLastError(const std::string& message);
}

struct dk_sparse_volume {
    std::vector<dk_volume_descriptor> volumes;
    std::vector<dk_volume_brick_descriptor> bricks;
    std::vector<dk_volume_brick_sample> samples;
    std::vector<dk_volume_brick_grid> grids;
    std::vector<uint32_t> gridIndices;
};

namespace {

struct Field {
    float distance;
    uint32_t material, secondary;
    float blend;
};

// combine (SDFModel.swift:511-570) without material fields / attributes.
inline Field combine(const Field& cur, float d, uint32_t mat, float smoothRadius) {
    if (!std::isfinite(cur.distance)) return {d, mat, mat, 0.0f};
    float radius = std::fmax(smoothRadius, 0.0f);
    if (!(radius > 1e-6f)) {
        if (d < cur.distance) return {d, mat, mat, 0.0f};
        return cur;
    }
    float h = std::fmin(std::fmax(0.5f + 0.5f * (d - cur.distance) / radius, 0.0f), 1.0f);
    float distance = (d + (cur.distance - d) * h) - radius * h * (1.0f - h);
    float w = 1.0f - h;
    if (w <= 0.001f) return {distance, cur.material, cur.secondary, cur.blend};
    if (w >= 0.999f) return {distance, mat, mat, 0.0f};
    return {distance, cur.material, mat, w};
}

// The same chain on distances only (monotone in both arguments).
inline float combineDistance(float cur, float d, float smoothRadius) {
    if (!std::isfinite(cur)) return d;
    float radius = std::fmax(smoothRadius, 0.0f);
    if (!(radius > 1e-6f)) return d < cur ? d : cur;
    float h = std::fmin(std::fmax(0.5f + 0.5f * (d - cur) / radius, 0.0f), 1.0f);
    return (d + (cur - d) * h) - radius * h * (1.0f - h);
}

inline float sphereDistance(const dk_sdf_sphere& s, float x, float y, float z) {
    float lx = x - s.center[0], ly = y - s.center[1], lz = z - s.center[2];
    return std::sqrt(lx * lx + ly * ly + lz * lz) - s.radius;
}

// The virtual grid of one build.
struct BakeGrid {
    int dims[3], bs[3], grid[3];
    float bmin[3], ext[3];
    float band;
    uint32_t fallback;
};

constexpr int kOverlap = 2;  // stored samples beyond the brick core on each side

// Core and stored sample ranges of the brick of cell `c` (z-y-x order).
__host__ __device__ inline void brickRange(const BakeGrid& G, size_t c, int core[3], int coreDims[3], int so[3],
                                           int sd[3]) {
    int cell[3] = {(int)(c % (size_t)G.grid[0]), (int)((c / (size_t)G.grid[0]) % (size_t)G.grid[1]),
                   (int)(c / ((size_t)G.grid[0] * G.grid[1]))};
    for (int a = 0; a < 3; ++a) {
        core[a] = cell[a] * G.bs[a];
        coreDims[a] = G.bs[a] < G.dims[a] - core[a] ? G.bs[a] : G.dims[a] - core[a];
        so[a] = core[a] - kOverlap > 0 ? core[a] - kOverlap : 0;
        int end = core[a] + coreDims[a] + kOverlap < G.dims[a] ? core[a] + coreDims[a] + kOverlap : G.dims[a];
        sd[a] = end - so[a];
    }
}

// ---- device restatements: the same operations, explicitly rounded, so a
// GPU build equals the host build bit for bit (the host side is compiled
// without FMA contraction).
__device__ __forceinline__ float dPos(const BakeGrid& G, int a, int i) {  // samplePosition
    float w = G.dims[a] == 1 ? 0.0f : __fdiv_rn((float)i, (float)(G.dims[a] - 1));
    return __fadd_rn(G.bmin[a], __fmul_rn(G.ext[a], w));
}

__device__ __forceinline__ float dSmoothH(float cur, float d, float radius) {
    return fminf(fmaxf(__fadd_rn(0.5f, __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(d, cur)), radius)), 0.0f), 1.0f);
}

__device__ __forceinline__ float dSmoothMin(float cur, float d, float radius, float h) {
    return __fsub_rn(__fadd_rn(d, __fmul_rn(__fsub_rn(cur, d), h)), __fmul_rn(__fmul_rn(radius, h), __fsub_rn(1.0f, h)));
}

__device__ __forceinline__ float dCombineDistance(float cur, float d, float smoothRadius) {
    if (!isfinite(cur)) return d;
    float radius = fmaxf(smoothRadius, 0.0f);
    if (!(radius > 1e-6f)) return d < cur ? d : cur;
    return dSmoothMin(cur, d, radius, dSmoothH(cur, d, radius));
}

__device__ __forceinline__ dk_volume_brick_sample dCombine(const dk_volume_brick_sample& cur, float d, uint32_t mat,
                                                           float smoothRadius) {
    if (!isfinite(cur.distance)) return {d, mat, mat, 0.0f};
    float radius = fmaxf(smoothRadius, 0.0f);
    if (!(radius > 1e-6f)) {
        if (d < cur.distance) return {d, mat, mat, 0.0f};
        return cur;
    }
    float h = dSmoothH(cur.distance, d, radius);
    float distance = dSmoothMin(cur.distance, d, radius, h);
    float w = __fsub_rn(1.0f, h);
    if (w <= 0.001f) return {distance, cur.material_a, cur.material_b, cur.material_blend};
    if (w >= 0.999f) return {distance, mat, mat, 0.0f};
    return {distance, cur.material_a, mat, w};
}

__device__ __forceinline__ float dSphereDistance(const dk_sdf_sphere& s, float x, float y, float z) {
    float lx = __fsub_rn(x, s.center[0]), ly = __fsub_rn(y, s.center[1]), lz = __fsub_rn(z, s.center[2]);
    return __fsub_rn(__fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(lx, lx), __fmul_rn(ly, ly)), __fmul_rn(lz, lz))),
                     s.radius);
}

// Interval pre-filter of every cell: 1 when the union's bounds over the
// brick's stored-sample box can reach the narrow band.
__global__ void k_sdf_classify(const dk_sdf_sphere* sp, uint32_t n, BakeGrid G, size_t cells, uint8_t* flags) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < cells; c += (size_t)gridDim.x * blockDim.x) {
        int core[3], coreDims[3], so[3], sd[3];
        brickRange(G, c, core, coreDims, so, sd);
        float lo3[3], hi3[3];
        for (int a = 0; a < 3; ++a) {
            lo3[a] = dPos(G, a, so[a]);
            hi3[a] = dPos(G, a, so[a] + sd[a] - 1);
        }
        float curLo = FLT_MAX, curHi = FLT_MAX;
        for (uint32_t i = 0; i < n; ++i) {
            const dk_sdf_sphere s = sp[i];
            float near2 = 0.0f, far2 = 0.0f;
            for (int a = 0; a < 3; ++a) {
                float cpa = s.center[a];
                float dn = fmaxf(fmaxf(__fsub_rn(lo3[a], cpa), __fsub_rn(cpa, hi3[a])), 0.0f);
                float df = fmaxf(fabsf(__fsub_rn(lo3[a], cpa)), fabsf(__fsub_rn(hi3[a], cpa)));
                near2 = __fadd_rn(near2, __fmul_rn(dn, dn));
                far2 = __fadd_rn(far2, __fmul_rn(df, df));
            }
            float dlo = __fsub_rn(__fsqrt_rn(near2), s.radius), dhi = __fsub_rn(__fsqrt_rn(far2), s.radius);
            curLo = dCombineDistance(curLo, dlo, s.smooth_union_radius);
            curHi = dCombineDistance(curHi, dhi, s.smooth_union_radius);
        }
        const float margin = 1e-4f;
        flags[c] = (curLo > __fadd_rn(G.band, margin) || curHi < __fsub_rn(-G.band, margin)) ? 0u : 1u;
    }
}

// One block per candidate brick: every stored sample (sampleField), and the
// brick's distance range.  cand[k] = (origin xyz, first output sample),
// candDims[k] = (dims xyz, sample count).
__global__ void __launch_bounds__(256) k_sdf_sample(const dk_sdf_sphere* sp, uint32_t n, BakeGrid G,
                                                    const uint4* cand, const uint4* candDims,
                                                    dk_volume_brick_sample* out, float2* range) {
    __shared__ float smin[8], smax[8];
    const uint4 o = cand[blockIdx.x], d = candDims[blockIdx.x];
    float mn = FLT_MAX, mx = -FLT_MAX;
    for (uint32_t k = threadIdx.x; k < d.w; k += blockDim.x) {
        uint32_t x = k % d.x, y = (k / d.x) % d.y, z = k / (d.x * d.y);
        float px = dPos(G, 0, (int)(o.x + x)), py = dPos(G, 1, (int)(o.y + y)), pz = dPos(G, 2, (int)(o.z + z));
        dk_volume_brick_sample f{FLT_MAX, G.fallback, G.fallback, 0.0f};  // sampleField starts at the largest float
        for (uint32_t i = 0; i < n; ++i) f = dCombine(f, dSphereDistance(sp[i], px, py, pz), sp[i].material,
                                                      sp[i].smooth_union_radius);
        out[o.w + k] = f;
        mn = fminf(mn, f.distance);
        mx = fmaxf(mx, f.distance);
    }
    for (int s = 16; s > 0; s >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, s));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, s));
    }
    if ((threadIdx.x & 31) == 0) {
        smin[threadIdx.x >> 5] = mn;
        smax[threadIdx.x >> 5] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            mn = fminf(mn, smin[w]);
            mx = fmaxf(mx, smax[w]);
        }
        range[blockIdx.x] = make_float2(mn, mx);
    }
}

}  // namespace

namespace {

struct Brick {
    int origin[3], dims[3], core[3], coreDims[3];
    const dk_volume_brick_sample* samples;      // dims product samples, x fastest
    std::vector<dk_volume_brick_sample> own;  // host build: the storage of `samples`
};

int setupGrid(const dk_sdf_sphere* spheres, uint32_t sphereCount, const dk_sparse_volume_settings* st,
              dk_sparse_volume** out, BakeGrid& G, size_t& cellCount) {
    if (!out || !st || (sphereCount > 0 && !spheres)) {
        dk::setLastError("sparse volume build: null argument");
        return DK_ERROR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    if (sphereCount == 0) {
        dk::setLastError("Invalid render scene: an SDF model needs at least one primitive.");
        return DK_ERROR_INVALID_SCENE;
    }
    for (int a = 0; a < 3; ++a) {
        G.dims[a] = (int)st->resolution[a];
        G.bs[a] = (int)std::max(1u, st->brick_size[a]);
        G.bmin[a] = st->bounds_min[a];
        G.ext[a] = st->bounds_max[a] - st->bounds_min[a];
        if (G.dims[a] < 2 || !(G.ext[a] > 0.0f)) {
            dk::setLastError("Invalid render scene: sparse distance volume needs >= 2 samples and positive extent per axis.");
            return DK_ERROR_INVALID_SCENE;
        }
        G.grid[a] = (G.dims[a] + G.bs[a] - 1) / G.bs[a];
    }
    G.band = st->narrow_band;
    G.fallback = spheres[0].material;
    cellCount = (size_t)G.grid[0] * G.grid[1] * G.grid[2];
    return DK_OK;
}

// gpuVolumeBricks + appendSparseVolumeDescriptor over the kept bricks, one
// per cell at most, in cell (z-y-x) order.
dk_sparse_volume* assemble(const BakeGrid& G, size_t cellCount, const std::vector<Brick*>& perCell,
                           const dk_sparse_volume_settings* st) {
    dk_sparse_volume* v = new dk_sparse_volume();
    // Grid + macro occupancy (SparseVolumeGPUEncoding.swift:67-103).
    const int macro = 4;
    int mdim[3];
    for (int a = 0; a < 3; ++a) mdim[a] = (G.grid[a] + macro - 1) / macro;
    size_t macroCount = (size_t)mdim[0] * mdim[1] * mdim[2];
    v->gridIndices.assign(cellCount, 0xffffffffu);
    v->gridIndices.resize(cellCount + macroCount, 0u);
    dk_volume_brick_grid g;
    g.dimensions_and_index_offset = {(uint32_t)G.grid[0], (uint32_t)G.grid[1], (uint32_t)G.grid[2], 0u};
    g.brick_size_and_volume = {(uint32_t)G.bs[0], (uint32_t)G.bs[1], (uint32_t)G.bs[2], 0u};
    g.macro_dimensions_and_index_offset = {(uint32_t)mdim[0], (uint32_t)mdim[1], (uint32_t)mdim[2], (uint32_t)cellCount};
    g.macro_size_and_reserved = {(uint32_t)macro, (uint32_t)macro, (uint32_t)macro, 0u};
    v->grids.push_back(g);
    size_t total = 0;
    for (const Brick* b : perCell)
        if (b) total += (size_t)b->dims[0] * b->dims[1] * b->dims[2];
    v->samples.reserve(total);
    const bool fp16 = st->fp16_distances != 0;
    float den[3];
    for (int a = 0; a < 3; ++a) den[a] = (float)std::max(G.dims[a] - 1, 1);
    for (size_t c = 0; c < cellCount; ++c) {
        const Brick* b = perCell[c];
        if (!b) continue;
        uint32_t brickIndex = (uint32_t)v->bricks.size();
        uint32_t sampleOffset = (uint32_t)v->samples.size();
        const size_t n = (size_t)b->dims[0] * b->dims[1] * b->dims[2];
        v->samples.insert(v->samples.end(), b->samples, b->samples + n);
        float dmin = FLT_MAX, dmax = -FLT_MAX;
        for (size_t k = sampleOffset; k < sampleOffset + n; ++k) {
            float& d = v->samples[k].distance;
            if (fp16) d = __half2float(__float2half_rn(d));  // FP16 storage: the stored value is the rounded one
            dmin = std::fmin(dmin, d);
            dmax = std::fmax(dmax, d);
        }
        dk_volume_brick_descriptor d;
        float cmin[3], cmax[3], smin[3], smax[3];
        for (int a = 0; a < 3; ++a) {  // brickCoreLocalBounds / brickSampleLocalBounds (:578-653)
            float gmn = std::fmax((float)b->core[a] - 0.5f, 0.0f);
            float gmx = std::fmin((float)(b->core[a] + b->coreDims[a] - 1) + 0.5f, den[a]);
            cmin[a] = G.bmin[a] + G.ext[a] * (gmn / den[a]);
            cmax[a] = G.bmin[a] + G.ext[a] * (gmx / den[a]);
            smin[a] = G.bmin[a] + G.ext[a] * ((float)b->origin[a] / den[a]);
            smax[a] = G.bmin[a] + G.ext[a] * ((float)(b->origin[a] + b->dims[a] - 1) / den[a]);
        }
        d.world_bounds_min = {cmin[0], cmin[1], cmin[2], 0.0f};
        d.world_bounds_max = {cmax[0], cmax[1], cmax[2], 0.0f};
        d.local_bounds_min = d.world_bounds_min;
        d.local_bounds_max = d.world_bounds_max;
        d.sample_bounds_min = {smin[0], smin[1], smin[2], dmin};
        d.sample_bounds_max = {smax[0], smax[1], smax[2], dmax};
        d.grid_origin_and_volume = {(uint32_t)b->origin[0], (uint32_t)b->origin[1], (uint32_t)b->origin[2], 0u};
        d.dimensions_and_sample_offset = {(uint32_t)b->dims[0], (uint32_t)b->dims[1], (uint32_t)b->dims[2],
                                          sampleOffset};
        v->bricks.push_back(d);
        int cell[3] = {b->core[0] / G.bs[0], b->core[1] / G.bs[1], b->core[2] / G.bs[2]};
        v->gridIndices[(size_t)cell[0] + (size_t)cell[1] * G.grid[0] + (size_t)cell[2] * G.grid[0] * G.grid[1]] =
            brickIndex;
        int m[3] = {cell[0] / macro, cell[1] / macro, cell[2] / macro};
        v->gridIndices[cellCount + (size_t)m[0] + (size_t)m[1] * mdim[0] + (size_t)m[2] * mdim[0] * mdim[1]] = 1u;
    }
    // appendSparseVolumeDescriptor (VolumeGPUEncoding.swift:184-243), identity transform.
    dk_volume_descriptor vd;
    std::memset(&vd, 0, sizeof(vd));
    vd.world_bounds_min = {st->bounds_min[0], st->bounds_min[1], st->bounds_min[2], 0.0f};
    vd.world_bounds_max = {st->bounds_max[0], st->bounds_max[1], st->bounds_max[2], 0.0f};
    vd.local_bounds_min = vd.world_bounds_min;
    vd.local_bounds_max = vd.world_bounds_max;
    vd.dimensions = {(uint32_t)G.dims[0], (uint32_t)G.dims[1], (uint32_t)G.dims[2], st->volume_material};
    vd.metadata = {0u, st->object_id, st->primitive_id, 1u};
    vd.material_program = {0xffffffffu, 0u, 0u, 0u};
    for (int c = 0; c < 4; ++c) {
        float col[4] = {0, 0, 0, 0};
        col[c] = 1.0f;
        vd.world_to_local[c] = {col[0], col[1], col[2], col[3]};
        vd.normal_transform[c] = {col[0], col[1], col[2], col[3]};
    }
    v->volumes.push_back(vd);
    return v;
}

}  // namespace

extern "C" {

int dk_build_sparse_sphere_volume(const dk_sdf_sphere* spheres, uint32_t sphereCount,
                                  const dk_sparse_volume_settings* st, dk_sparse_volume** out) {
    BakeGrid G;
    size_t cellCount = 0;
    int rc = setupGrid(spheres, sphereCount, st, out, G, cellCount);
    if (rc != DK_OK) return rc;
    const float band = G.band;
    // samplePosition (SDFModel.swift:452-464)
    auto pos = [&](int a, int i) {
        float w = G.dims[a] == 1 ? 0.0f : (float)i / (float)(G.dims[a] - 1);
        return G.bmin[a] + G.ext[a] * w;
    };
    std::vector<Brick*> perCell(cellCount, nullptr);
    std::atomic<size_t> next(0);
    auto worker = [&]() {
        for (;;) {
            size_t c = next.fetch_add(1);
            if (c >= cellCount) break;
            int core[3], coreDims[3], so[3], sd[3];
            brickRange(G, c, core, coreDims, so, sd);
            // Interval bound of the union over the stored samples' box.
            float lo3[3], hi3[3];
            for (int a = 0; a < 3; ++a) {
                lo3[a] = pos(a, so[a]);
                hi3[a] = pos(a, so[a] + sd[a] - 1);
            }
            float curLo = FLT_MAX, curHi = FLT_MAX;
            for (uint32_t i = 0; i < sphereCount; ++i) {
                const dk_sdf_sphere& s = spheres[i];
                float near2 = 0.0f, far2 = 0.0f;
                for (int a = 0; a < 3; ++a) {
                    float cpa = s.center[a];
                    float dn = std::fmax(std::fmax(lo3[a] - cpa, cpa - hi3[a]), 0.0f);
                    float df = std::fmax(std::fabs(lo3[a] - cpa), std::fabs(hi3[a] - cpa));
                    near2 += dn * dn;
                    far2 += df * df;
                }
                float dlo = std::sqrt(near2) - s.radius, dhi = std::sqrt(far2) - s.radius;
                curLo = combineDistance(curLo, dlo, s.smooth_union_radius);
                curHi = combineDistance(curHi, dhi, s.smooth_union_radius);
            }
            const float margin = 1e-4f;
            if (curLo > band + margin || curHi < -band - margin) continue;
            Brick* b = new Brick();
            for (int a = 0; a < 3; ++a) {
                b->origin[a] = so[a];
                b->dims[a] = sd[a];
                b->core[a] = core[a];
                b->coreDims[a] = coreDims[a];
            }
            size_t n = (size_t)sd[0] * sd[1] * sd[2];
            b->own.resize(n);
            float mn = FLT_MAX, mxv = -FLT_MAX;
            for (int z = 0; z < sd[2]; ++z)
                for (int y = 0; y < sd[1]; ++y)
                    for (int x = 0; x < sd[0]; ++x) {
                        float px = pos(0, so[0] + x), py = pos(1, so[1] + y), pz = pos(2, so[2] + z);
                        // sampleField (SDFModel.swift:466-498): starts at greatestFiniteMagnitude.
                        Field f{FLT_MAX, G.fallback, G.fallback, 0.0f};
                        for (uint32_t i = 0; i < sphereCount; ++i)
                            f = combine(f, sphereDistance(spheres[i], px, py, pz), spheres[i].material,
                                        spheres[i].smooth_union_radius);
                        b->own[(size_t)x + (size_t)y * sd[0] + (size_t)z * sd[0] * sd[1]] = {f.distance, f.material,
                                                                                            f.secondary, f.blend};
                        mn = std::fmin(mn, f.distance);
                        mxv = std::fmax(mxv, f.distance);
                    }
            // brickIntersectsNarrowBand (SDFModel.swift:505-507)
            if (!(mn <= band && mxv >= -band)) {
                delete b;
                continue;
            }
            b->samples = b->own.data();
            perCell[c] = b;
        }
    };
    unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
    *out = assemble(G, cellCount, perCell, st);
    for (Brick* b : perCell) delete b;
    return DK_OK;
}

// The same volume with the sampling on the current CUDA device: the interval
// pre-filter per cell (k_sdf_classify), then every stored sample of the
// surviving bricks, one block per brick (k_sdf_sample); the narrow-band test
// and the assembly run on the host.  Bit-identical to
// dk_build_sparse_sphere_volume.
int dk_bake_sparse_sphere_volume(const dk_sdf_sphere* spheres, uint32_t sphereCount,
                                 const dk_sparse_volume_settings* st, dk_sparse_volume** out) {
    BakeGrid G;
    size_t cellCount = 0;
    int rc = setupGrid(spheres, sphereCount, st, out, G, cellCount);
    if (rc != DK_OK) return rc;
    dk_sdf_sphere* dSp = nullptr;
    uint8_t* dFlags = nullptr;
    uint4 *dCand = nullptr, *dDims = nullptr;
    dk_volume_brick_sample* dOut = nullptr;
    float2* dRange = nullptr;
    std::string err;
    auto check = [&](cudaError_t e, const char* what) {
        if (e != cudaSuccess && err.empty()) err = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaSuccess;
    };
    std::vector<uint8_t> flags(cellCount);
    std::vector<uint4> cand, dims;
    std::vector<dk_volume_brick_sample> samples;
    std::vector<float2> range;
    std::vector<size_t> candCell;
    if (check(cudaMalloc(&dSp, sphereCount * sizeof(dk_sdf_sphere)), "cudaMalloc") &&
        check(cudaMemcpy(dSp, spheres, sphereCount * sizeof(dk_sdf_sphere), cudaMemcpyHostToDevice), "upload") &&
        check(cudaMalloc(&dFlags, cellCount), "cudaMalloc")) {
        int grid = (int)std::min<size_t>((cellCount + 255) / 256, 152 * 16);
        k_sdf_classify<<<grid, 256>>>(dSp, sphereCount, G, cellCount, dFlags);
        check(cudaGetLastError(), "classify launch");
        check(cudaMemcpy(flags.data(), dFlags, cellCount, cudaMemcpyDeviceToHost), "classify readback");
    }
    size_t total = 0;
    if (err.empty()) {
        for (size_t c = 0; c < cellCount; ++c) {
            if (!flags[c]) continue;
            int core[3], coreDims[3], so[3], sd[3];
            brickRange(G, c, core, coreDims, so, sd);
            uint32_t n = (uint32_t)sd[0] * sd[1] * sd[2];
            if (total + n > 0xffffffffull) {
                err = "sparse volume too large for 32-bit sample offsets";
                break;
            }
            cand.push_back(make_uint4(so[0], so[1], so[2], (uint32_t)total));
            dims.push_back(make_uint4(sd[0], sd[1], sd[2], n));
            candCell.push_back(c);
            total += n;
        }
    }
    if (err.empty() && !cand.empty()) {
        samples.resize(total);
        range.resize(cand.size());
        if (check(cudaMalloc(&dCand, cand.size() * sizeof(uint4)), "cudaMalloc") &&
            check(cudaMalloc(&dDims, dims.size() * sizeof(uint4)), "cudaMalloc") &&
            check(cudaMalloc(&dOut, total * sizeof(dk_volume_brick_sample)), "cudaMalloc") &&
            check(cudaMalloc(&dRange, range.size() * sizeof(float2)), "cudaMalloc") &&
            check(cudaMemcpy(dCand, cand.data(), cand.size() * sizeof(uint4), cudaMemcpyHostToDevice), "upload") &&
            check(cudaMemcpy(dDims, dims.data(), dims.size() * sizeof(uint4), cudaMemcpyHostToDevice), "upload")) {
            k_sdf_sample<<<(unsigned)cand.size(), 256>>>(dSp, sphereCount, G, dCand, dDims, dOut, dRange);
            check(cudaGetLastError(), "sample launch");
            check(cudaMemcpy(range.data(), dRange, range.size() * sizeof(float2), cudaMemcpyDeviceToHost), "readback");
            check(cudaMemcpy(samples.data(), dOut, total * sizeof(dk_volume_brick_sample), cudaMemcpyDeviceToHost),
                  "readback");
        }
    }
    cudaFree(dSp);
    cudaFree(dFlags);
    cudaFree(dCand);
    cudaFree(dDims);
    cudaFree(dOut);
    cudaFree(dRange);
    if (!err.empty()) {
        dk::setLastError("sparse volume bake: " + err);
        return DK_ERROR_COMMAND_FAILED;
    }
    std::vector<Brick> bricks(cand.size());
    std::vector<Brick*> perCell(cellCount, nullptr);
    for (size_t k = 0; k < cand.size(); ++k) {
        // brickIntersectsNarrowBand (SDFModel.swift:505-507)
        if (!(range[k].x <= G.band && range[k].y >= -G.band)) continue;
        Brick& b = bricks[k];
        int so[3], sd[3];
        brickRange(G, candCell[k], b.core, b.coreDims, so, sd);
        for (int a = 0; a < 3; ++a) {
            b.origin[a] = so[a];
            b.dims[a] = sd[a];
        }
        b.samples = samples.data() + cand[k].w;
        perCell[candCell[k]] = &b;
    }
    *out = assemble(G, cellCount, perCell, st);
    return DK_OK;
}

int dk_sparse_volume_view(const dk_sparse_volume* v, dk_scene* scene) {
    if (!v || !scene) {
        dk::setLastError("dk_sparse_volume_view: null argument");
        return DK_ERROR_INVALID_ARGUMENT;
    }
    scene->volumes = v->volumes.data();
    scene->volume_count = (uint32_t)v->volumes.size();
    scene->volume_bricks = v->bricks.data();
    scene->volume_brick_count = (uint32_t)v->bricks.size();
    scene->volume_brick_samples = v->samples.data();
    scene->volume_brick_sample_count = v->samples.size();
    scene->volume_brick_grids = v->grids.data();
    scene->volume_brick_grid_count = (uint32_t)v->grids.size();
    scene->volume_brick_grid_indices = v->gridIndices.data();
    scene->volume_brick_grid_index_count = v->gridIndices.size();
    return DK_OK;
}

int dk_sparse_volume_destroy(dk_sparse_volume* v) {
    delete v;
    return DK_OK;
}

}  // extern "C"
