// Plain-old-data views shared by the host side (dk_host.cu) and the kernels
// (dk_kernels.cu) of the sm_103a path tracer, plus the kernel launchers.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/denrim_cuda.h"

namespace dk {

constexpr uint32_t kNoSlot = 0xffffffffu;

// Device copy of the scene.  `isect` holds 3 x float4 per BVH leaf slot:
// (v0.xyz, reference slot), (v1 - v0, triangle index), (v2 - v0, flags with
// bit 0 = blocks shadow rays); `nodes` holds 4 x float4 per node: the x, y and
// z slabs of both child boxes and the two child references.
struct DevScene {
    const dk_triangle* tris;
    const dk_material* mats;
    const float4* isect;
    const float4* nodes;
    const dk_texture_descriptor* texdesc;
    const float4* texpix;
    const dk_light_record* lights;
    const float2* env;
    const uint32_t* env_guide;  // G + 1 entries: first index with cdf >= b / G (G a power of two)
    uint32_t tri_count, mat_count, node_count, texdesc_count;
    uint32_t light_count, env_count, env_tex_plus1, all_shadow_opaque;
    float env_intensity, env_rot_y, env_max_radiance;
    uint32_t env_guide_size;
    // Sparse distance volumes (GPUVolumeDescriptor with metadata.w == 1).
    const dk_volume_descriptor* volumes;
    const dk_volume_brick_descriptor* bricks;
    const dk_volume_brick_sample* brick_samples;
    const float* brick_dist;  // distance-only copy of brick_samples
    const dk_volume_brick_grid* brick_grids;
    const uint32_t* brick_grid_indices;
    uint64_t brick_sample_count, brick_grid_index_count;
    uint32_t volume_count, brick_count, brick_grid_count, volume_all_opaque;
};

// GPURenderConstants (PathTrace.metal:143-182) for one batch of samples.
struct DevParams {
    uint32_t width, height, max_bounces, transparent_background;
    uint32_t shows_env_bg, frame_seed, denoiser, pad0;
    float bg[3];
    float clamp;
    uint32_t tile_x, tile_y, tile_w, tile_h;
    uint32_t sample_begin, samples_in_batch, path_count, pad1;
    dk_camera cam, prev_cam;
};

// SoA path state of one batch ("wave") of `cap` paths.
struct Wave {
    float4* ray_o;     // origin
    float4* ray_d;     // direction
    float4* tp;        // throughput, w = previous BSDF pdf
    float4* rad;       // radiance, w = alpha
    uint2* rng;        // RNG state, flags (bit 0: primary hit found)
    float4* hit;       // t, triangle, u, v
    float4* nee_o;     // 3 slots x cap: shadow origin, w = max distance
    float4* nee_d;     // 3 slots x cap: shadow direction
    float4* nee_c;     // 3 slots x cap: unshadowed contribution, w = pdf divisor
    float4* nee_tp;    // throughput at NEE, w = slot mask
    uint32_t* q[2];    // active path queues (ping-pong)
    uint32_t* qs;      // paths with shadow queries
    uint32_t* qr;      // shadow rays: path << 2 | slot (3 x cap entries)
    uint32_t* qr2;     // shadow rays that need the layer walk (3 x cap entries)
    uint32_t* counts;  // [0], [1] queue lengths, [2] shadow paths, [3] shadow rays, [4] extend cursor,
                       // [5] shadow cursor, [6] layer-walk rays, [7] spare
    float4* aov;       // 4 x tile pixels: primary-hit record of the batch's last sample
    uint32_t cap;
    uint32_t pad;
};

struct alignas(32) D4 { double x, y, z, w; };

// Per-pixel accumulation of a session.
struct Accum {
    float4* sum;       // Kahan sum
    float4* comp;      // Kahan compensation
    D4* resolved;   // FP64 resolve of every completed 4096-sample block
    uint32_t* count;   // samples accumulated per pixel
    float4* aov;       // 6 planes: depth, normal, albedo, materialID, objectID, motion
};

// Host-side traversal BVH (dk_bvh.cu).
bool referenceSlots(const dk_scene* sc, std::vector<uint32_t>& slotOfTri, std::string& err);
int buildSahTraversal(const dk_scene* sc, const std::vector<uint32_t>& slotOfTri, const std::vector<uint8_t>& opaque,
                      std::vector<float4>& nodes, std::vector<float4>& isect, std::string& err);

cudaError_t launchGenerate(const DevScene& S, const DevParams& P, const Wave& W, int grid, cudaStream_t st);
cudaError_t launchExtend(const DevScene& S, const Wave& W, uint32_t sel, int grid, cudaStream_t st);
cudaError_t launchShade(const DevScene& S, const DevParams& P, const Wave& W, uint32_t bounce, uint32_t sel, int grid,
                        cudaStream_t st);
cudaError_t launchShadow(const DevScene& S, const DevParams& P, const Wave& W, int grid, cudaStream_t st);
cudaError_t launchResolve(const DevParams& P, const Wave& W, int grid, cudaStream_t st);
cudaError_t launchAovPrimary(const DevScene& S, const DevParams& P, const Wave& W, int grid, cudaStream_t st);
cudaError_t launchFinalize(const DevParams& P, const Wave& W, const Accum& A, uint32_t writeAov, int grid,
                           cudaStream_t st);
cudaError_t launchResolveBeauty(const Accum& A, uint32_t pixels, float4* out, int grid, cudaStream_t st);
cudaError_t buildEnvironmentTable(const float4* dPixels, uint32_t w, uint32_t h, float intensity, float maxR,
                                  double* dWeights, double* dPrefix, double* dBlockSums, float2* dOut, int grid,
                                  cudaStream_t st, double* hostTotal);

}  // namespace dk
