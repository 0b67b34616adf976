// Test infrastructure: host driver that runs the reference's own compute
// kernels `pathTraceKernel` (PathTrace.metal:5167-5586), `flatPreviewKernel`
// (:4728-4868) and `interactiveMaterialKernel` (:4870-5165) -- rewritten to C++
// by metal2cpp.py and compiled against metal_shim.hpp -- once per pixel and
// sample (the kernel DenrimRenderer.primaryPipeline picks for the quality,
// DenrimRenderer.swift:197-214),
// the way RenderSession.encodeNextSample dispatches it
// (RenderSession.swift:891-1007): GPURenderConstants filled from the settings,
// sampleIndex advanced per sample, the RGBA32F running-mean accumulation
// texture read and written by the kernel, AOVs written per sample.
// Pixels run in parallel on host threads; every pixel owns its texels.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

#include "../oracle_params.h"
#include "pathtrace_ref.cpp"

namespace {

using namespace mref;

static_assert(sizeof(GPUTriangle) == sizeof(dk_triangle), "GPUTriangle layout");
static_assert(sizeof(GPUMaterial) == sizeof(dk_material), "GPUMaterial layout");
static_assert(sizeof(GPUAccelerationNode) == sizeof(dk_bvh_node), "GPUAccelerationNode layout");
static_assert(sizeof(GPULightRecord) == sizeof(dk_light_record), "GPULightRecord layout");
static_assert(sizeof(GPUEnvironmentSample) == sizeof(dk_environment_sample), "GPUEnvironmentSample layout");
static_assert(sizeof(GPUVolumeDescriptor) == sizeof(dk_volume_descriptor), "GPUVolumeDescriptor layout");
static_assert(sizeof(GPUVolumeBrickDescriptor) == sizeof(dk_volume_brick_descriptor), "brick layout");
static_assert(sizeof(GPUVolumeBrickSample) == sizeof(dk_volume_brick_sample), "brick sample layout");
static_assert(sizeof(GPUVolumeBrickGrid) == sizeof(dk_volume_brick_grid), "brick grid layout");
static_assert(sizeof(GPUCamera) == sizeof(dk_camera), "GPUCamera layout");

// Stand-in for the reference's placeholder buffers bound when a count is 0.
alignas(64) static unsigned char g_empty[4096];

template <class T> const T* buf(std::nullptr_t) { return reinterpret_cast<const T*>(g_empty); }
template <class T, class U> const T* buf(const U* p) {
    return p ? reinterpret_cast<const T*>(p) : reinterpret_cast<const T*>(g_empty);
}

}  // namespace

extern "C" {

// Number of SDF traversal counters the reference kernel keeps
// (sdfCounterDenseVolumeTests .. sdfCounterShadowSceneQueries).
uint32_t ref_sdf_counter_count(void) { return 13u; }

// Renders samples [sample_begin, sample_begin + sample_count) of the tile in
// `params` (or of the listed pixels) with the reference kernel.  `accum` is the
// RGBA32F accumulation texture (W*H*4 floats), `aov` six W*H*4 float planes
// (depth, normal, albedo, material ID, object ID, motion vector), `sdf_counters`
// 13 counters or null (null disables sdfTraversalStatsEnabled).  `threads` <= 0
// uses every hardware thread.  Returns 0 on success, 1 for a bad argument, 2
// for an empty image and 4 when a listed pixel lies outside the image
// (nothing is written then).
// `quality` is RenderSettings.shaderQualityLevel: 0 preview, 1 interactive,
// 2 final (RenderSettings.swift:96-105).
int ref_render_quality(int quality, const dk_scene* scene, const oracle_params* p, uint32_t sample_begin,
                       uint32_t sample_count, const uint32_t* pixel_list, uint32_t pixel_list_count, int threads,
                       float* accum, float* aov, uint32_t* sdf_counters) {
    if (!scene || !p || !accum || !aov || quality < 0 || quality > 2) return 1;
    const uint32_t W = p->width, H = p->height;
    GPURenderConstants base{};
    base.width = W;
    base.height = H;
    base.triangleCount = scene->triangle_count;
    base.volumeCount = scene->volume_count;
    base.materialCount = scene->material_count;
    base.maxBounces = std::max(1u, p->max_bounces);
    base.renderQuality = (uint)quality;
    base.frameSeed = p->frame_seed;
    base.accelerationNodeCount = scene->node_count;
    base.transparentBackground = p->transparent_background;
    base.showsEnvironmentBackground = p->shows_environment_background;
    base.lightCount = scene->light_count;
    base.environmentTextureIndexPlusOne = scene->environment_texture_index_plus_one;
    base.environmentDistributionCount = scene->environment_sample_count;
    base.environmentIntensity = scene->environment_intensity;
    base.environmentRotationY = scene->environment_rotation_y;
    base.environmentMaxRadiance = scene->environment_max_radiance;
    base.sampleRadianceClamp = p->sample_radiance_clamp;
    base.backgroundColor = float4(p->background_color[0], p->background_color[1], p->background_color[2], 1.0f);
    base.volumeBrickCount = scene->volume_brick_count;
    base.volumeBrickSampleCount = (uint)scene->volume_brick_sample_count;
    base.volumeBrickGridCount = scene->volume_brick_grid_count;
    base.volumeBrickGridIndexCount = (uint)scene->volume_brick_grid_index_count;
    base.denoiserEnabled = p->denoiser_enabled;
    base.sdfTraversalStatsEnabled = sdf_counters ? 1u : 0u;
    base.tileX = p->tile_x;
    base.tileY = p->tile_y;
    base.tileWidth = p->tile_w;
    base.tileHeight = p->tile_h;

    GPUCamera camera, previous;
    std::memcpy(&camera, &p->camera, sizeof camera);
    std::memcpy(&previous, &p->previous_camera, sizeof previous);

    const size_t plane = (size_t)W * H;
    texture2d<float, access::read_write> accumulation{reinterpret_cast<float4*>(accum), W, H};
    texture2d<float, access::write> planes[6];
    for (int i = 0; i < 6; ++i) planes[i] = {reinterpret_cast<float4*>(aov) + plane * i, W, H};

    std::vector<atomic_uint> counters(13);
    for (auto& c : counters) c.value.store(0);

    if (W == 0 || H == 0) return 2;
    std::vector<uint32_t> pixels;
    if (pixel_list) {
        // Every listed pixel must lie in the W*H image.  (The kernels skip a
        // pixel outside the tile or the image themselves.)
        const uint64_t npix = (uint64_t)W * H;
        for (uint32_t i = 0; i < pixel_list_count; ++i)
            if (pixel_list[i] >= npix) return 4;
        pixels.assign(pixel_list, pixel_list + pixel_list_count);
    } else {
        for (uint32_t y = 0; y < p->tile_h; ++y)
            for (uint32_t x = 0; x < p->tile_w; ++x) pixels.push_back((p->tile_y + y) * W + p->tile_x + x);
    }

    unsigned nthreads = threads > 0 ? (unsigned)threads : std::max(1u, std::thread::hardware_concurrency());
    std::atomic<size_t> next{0};
    auto worker = [&]() {
        GPURenderConstants c = base;
        for (;;) {
            size_t begin = next.fetch_add(64);
            if (begin >= pixels.size()) break;
            size_t end = std::min(pixels.size(), begin + 64);
            for (size_t i = begin; i < end; ++i) {
                uint32_t px = pixels[i] % W, py = pixels[i] / W;
                uint2 gid(px - p->tile_x, py - p->tile_y);
                for (uint32_t s = 0; s < sample_count; ++s) {
                    c.sampleIndex = sample_begin + s;
                    auto kernel = quality == 2 ? pathTraceKernel : (quality == 1 ? interactiveMaterialKernel
                                                                                 : flatPreviewKernel);
                    kernel(accumulation, planes[0], planes[1], planes[2], planes[3], planes[4], planes[5],
                                    c, camera, buf<GPUTriangle>(scene->triangles),
                                    buf<GPUMaterial>(scene->materials), buf<GPUAccelerationNode>(scene->nodes),
                                    buf<uint>(scene->primitive_indices), previous,
                                    buf<GPUTextureDescriptor>(scene->texture_descriptors),
                                    buf<float4>(scene->texture_pixels), buf<GPULightRecord>(scene->lights),
                                    buf<GPUEnvironmentSample>(scene->environment_samples),
                                    buf<GPUVolumeDescriptor>(scene->volumes), buf<GPUVolumeSample>(nullptr),
                                    buf<GPUVolumeBrickDescriptor>(scene->volume_bricks),
                                    buf<GPUVolumeBrickSample>(scene->volume_brick_samples),
                                    buf<GPUVolumeAttributeDescriptor>(nullptr), buf<float4>(nullptr),
                                    buf<GPUVolumeAttributeDescriptor>(nullptr), buf<float4>(nullptr),
                                    buf<GPUAccelerationNode>(nullptr), buf<uint>(nullptr),
                                    buf<GPUVolumeBrickGrid>(scene->volume_brick_grids),
                                    buf<uint>(scene->volume_brick_grid_indices),
                                    buf<GPUVolumeMaterialFieldSample>(nullptr),
                                    sdf_counters ? counters.data() : nullptr,
                                    buf<GPUMaterialProgramDescriptor>(nullptr),
                                    buf<GPUMaterialProgramOperation>(nullptr), gid);
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nthreads; ++t) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
    if (sdf_counters)
        for (int i = 0; i < 13; ++i) sdf_counters[i] += counters[i].value.load();
    return 0;
}

int ref_render(const dk_scene* scene, const oracle_params* p, uint32_t sample_begin, uint32_t sample_count,
               const uint32_t* pixel_list, uint32_t pixel_list_count, int threads, float* accum, float* aov,
               uint32_t* sdf_counters) {
    return ref_render_quality(2, scene, p, sample_begin, sample_count, pixel_list, pixel_list_count, threads, accum,
                              aov, sdf_counters);
}

}  // extern "C"
