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

}  // namespace

extern "C" {

int dk_build_sparse_sphere_volume(const dk_sdf_sphere* spheres, uint32_t sphereCount,
                                  const dk_sparse_volume_settings* st, dk_sparse_volume** out) {
    if (!out || !st || (sphereCount > 0 && !spheres)) {
        dk::setLastError("dk_build_sparse_sphere_volume: null argument");
        return DK_ERROR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    if (sphereCount == 0) {
        dk::setLastError("Invalid render scene: an SDF model needs at least one primitive.");
        return DK_ERROR_INVALID_SCENE;
    }
    int dims[3], bs[3];
    float bmin[3], ext[3];
    for (int a = 0; a < 3; ++a) {
        dims[a] = (int)st->resolution[a];
        bs[a] = (int)std::max(1u, st->brick_size[a]);
        bmin[a] = st->bounds_min[a];
        ext[a] = st->bounds_max[a] - st->bounds_min[a];
        if (dims[a] < 2 || !(ext[a] > 0.0f)) {
            dk::setLastError("Invalid render scene: sparse distance volume needs >= 2 samples and positive extent per axis.");
            return DK_ERROR_INVALID_SCENE;
        }
    }
    const float band = st->narrow_band;
    const float defaultDistance = std::fmax(band, 1.0f);
    const uint32_t fallback = spheres[0].material;
    // samplePosition (SDFModel.swift:452-464)
    auto pos = [&](int a, int i) {
        float w = dims[a] == 1 ? 0.0f : (float)i / (float)(dims[a] - 1);
        return bmin[a] + ext[a] * w;
    };
    int grid[3];
    for (int a = 0; a < 3; ++a) grid[a] = (dims[a] + bs[a] - 1) / bs[a];
    const size_t cellCount = (size_t)grid[0] * grid[1] * grid[2];

    struct Brick {
        int origin[3], dims[3], core[3], coreDims[3];
        std::vector<Field> samples;
    };
    std::vector<std::vector<Brick>> perCell(cellCount);
    std::atomic<size_t> next(0);
    const int overlap = 2;
    auto worker = [&]() {
        for (;;) {
            size_t c = next.fetch_add(1);
            if (c >= cellCount) break;
            int cz = (int)(c / ((size_t)grid[0] * grid[1]));
            int cy = (int)((c / grid[0]) % grid[1]);
            int cx = (int)(c % grid[0]);
            int core[3] = {cx * bs[0], cy * bs[1], cz * bs[2]};
            int coreDims[3], so[3], sd[3];
            for (int a = 0; a < 3; ++a) {
                coreDims[a] = std::min(bs[a], dims[a] - core[a]);
                so[a] = std::max(core[a] - overlap, 0);
                int end = std::min(core[a] + coreDims[a] + overlap, dims[a]);
                sd[a] = end - so[a];
            }
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
            Brick b;
            for (int a = 0; a < 3; ++a) {
                b.origin[a] = so[a];
                b.dims[a] = sd[a];
                b.core[a] = core[a];
                b.coreDims[a] = coreDims[a];
            }
            size_t n = (size_t)sd[0] * sd[1] * sd[2];
            b.samples.assign(n, Field{defaultDistance, fallback, fallback, 0.0f});
            float mn = FLT_MAX, mxv = -FLT_MAX;
            for (int z = 0; z < sd[2]; ++z)
                for (int y = 0; y < sd[1]; ++y)
                    for (int x = 0; x < sd[0]; ++x) {
                        float px = pos(0, so[0] + x), py = pos(1, so[1] + y), pz = pos(2, so[2] + z);
                        // sampleField (SDFModel.swift:466-498): starts at greatestFiniteMagnitude.
                        Field f{FLT_MAX, fallback, fallback, 0.0f};
                        for (uint32_t i = 0; i < sphereCount; ++i)
                            f = combine(f, sphereDistance(spheres[i], px, py, pz), spheres[i].material,
                                        spheres[i].smooth_union_radius);
                        b.samples[(size_t)x + (size_t)y * sd[0] + (size_t)z * sd[0] * sd[1]] = f;
                        mn = std::fmin(mn, f.distance);
                        mxv = std::fmax(mxv, f.distance);
                    }
            // brickIntersectsNarrowBand (SDFModel.swift:505-507)
            if (!(mn <= band && mxv >= -band)) continue;
            perCell[c].push_back(std::move(b));
        }
    };
    unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();

    dk_sparse_volume* v = new dk_sparse_volume();
    // Grid + macro occupancy (SparseVolumeGPUEncoding.swift:67-103).
    const int macro = 4;
    int mdim[3];
    for (int a = 0; a < 3; ++a) mdim[a] = (grid[a] + macro - 1) / macro;
    size_t macroCount = (size_t)mdim[0] * mdim[1] * mdim[2];
    v->gridIndices.assign(cellCount, 0xffffffffu);
    v->gridIndices.resize(cellCount + macroCount, 0u);
    dk_volume_brick_grid g;
    g.dimensions_and_index_offset = {(uint32_t)grid[0], (uint32_t)grid[1], (uint32_t)grid[2], 0u};
    g.brick_size_and_volume = {(uint32_t)bs[0], (uint32_t)bs[1], (uint32_t)bs[2], 0u};
    g.macro_dimensions_and_index_offset = {(uint32_t)mdim[0], (uint32_t)mdim[1], (uint32_t)mdim[2], (uint32_t)cellCount};
    g.macro_size_and_reserved = {(uint32_t)macro, (uint32_t)macro, (uint32_t)macro, 0u};
    v->grids.push_back(g);
    float den[3];
    for (int a = 0; a < 3; ++a) den[a] = (float)std::max(dims[a] - 1, 1);
    // Bricks in the reference's z-y-x build order (cells are visited in that order).
    for (size_t c = 0; c < cellCount; ++c) {
        for (Brick& b : perCell[c]) {
            uint32_t brickIndex = (uint32_t)v->bricks.size();
            uint32_t sampleOffset = (uint32_t)v->samples.size();
            float dmin = FLT_MAX, dmax = -FLT_MAX;
            for (const Field& f : b.samples) {
                v->samples.push_back({f.distance, f.material, f.secondary, f.blend});
                dmin = std::fmin(dmin, f.distance);
                dmax = std::fmax(dmax, f.distance);
            }
            dk_volume_brick_descriptor d;
            float cmin[3], cmax[3], smin[3], smax[3];
            for (int a = 0; a < 3; ++a) {  // brickCoreLocalBounds / brickSampleLocalBounds (:578-653)
                float gmn = std::fmax((float)b.core[a] - 0.5f, 0.0f);
                float gmx = std::fmin((float)(b.core[a] + b.coreDims[a] - 1) + 0.5f, den[a]);
                cmin[a] = bmin[a] + ext[a] * (gmn / den[a]);
                cmax[a] = bmin[a] + ext[a] * (gmx / den[a]);
                smin[a] = bmin[a] + ext[a] * ((float)b.origin[a] / den[a]);
                smax[a] = bmin[a] + ext[a] * ((float)(b.origin[a] + b.dims[a] - 1) / den[a]);
            }
            d.world_bounds_min = {cmin[0], cmin[1], cmin[2], 0.0f};
            d.world_bounds_max = {cmax[0], cmax[1], cmax[2], 0.0f};
            d.local_bounds_min = d.world_bounds_min;
            d.local_bounds_max = d.world_bounds_max;
            d.sample_bounds_min = {smin[0], smin[1], smin[2], dmin};
            d.sample_bounds_max = {smax[0], smax[1], smax[2], dmax};
            d.grid_origin_and_volume = {(uint32_t)b.origin[0], (uint32_t)b.origin[1], (uint32_t)b.origin[2], 0u};
            d.dimensions_and_sample_offset = {(uint32_t)b.dims[0], (uint32_t)b.dims[1], (uint32_t)b.dims[2], sampleOffset};
            v->bricks.push_back(d);
            int cell[3] = {b.core[0] / bs[0], b.core[1] / bs[1], b.core[2] / bs[2]};
            v->gridIndices[(size_t)cell[0] + (size_t)cell[1] * grid[0] + (size_t)cell[2] * grid[0] * grid[1]] = brickIndex;
            int m[3] = {cell[0] / macro, cell[1] / macro, cell[2] / macro};
            v->gridIndices[cellCount + (size_t)m[0] + (size_t)m[1] * mdim[0] + (size_t)m[2] * mdim[0] * mdim[1]] = 1u;
        }
    }
    // appendSparseVolumeDescriptor (VolumeGPUEncoding.swift:184-243), identity transform.
    dk_volume_descriptor vd;
    std::memset(&vd, 0, sizeof(vd));
    vd.world_bounds_min = {st->bounds_min[0], st->bounds_min[1], st->bounds_min[2], 0.0f};
    vd.world_bounds_max = {st->bounds_max[0], st->bounds_max[1], st->bounds_max[2], 0.0f};
    vd.local_bounds_min = vd.world_bounds_min;
    vd.local_bounds_max = vd.world_bounds_max;
    vd.dimensions = {(uint32_t)dims[0], (uint32_t)dims[1], (uint32_t)dims[2], st->volume_material};
    vd.metadata = {0u, st->object_id, st->primitive_id, 1u};
    vd.material_program = {0xffffffffu, 0u, 0u, 0u};
    for (int c = 0; c < 4; ++c) {
        float col[4] = {0, 0, 0, 0};
        col[c] = 1.0f;
        vd.world_to_local[c] = {col[0], col[1], col[2], col[3]};
        vd.normal_transform[c] = {col[0], col[1], col[2], col[3]};
    }
    v->volumes.push_back(vd);
    *out = v;
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
