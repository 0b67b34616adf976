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
constexpr uint32_t kSortBins = 256;      // shading-order keys: 0 miss, 1 + material ID (< 254), 255 other
constexpr uint32_t kLiveBlock = 4096;    // paths per block of the survivor compaction (256 threads x 16)
constexpr uint32_t kRecLayers = 4;       // non-opaque layers the any-hit pass records per shadow ray
constexpr uint32_t kTraversalStack = 32; // groups on the 8-wide traversal stack (bounds the tree depth)

// Device copy of the scene.  `isect` holds 3 x float4 per BVH leaf slot:
// (v0.xyz, reference slot), (v1 - v0, triangle index), (v2 - v0, flags with
// bit 0 = blocks shadow rays under the scene's own materials and bits 8..15 =
// min(material ID, 255)); `nodes` holds the traversal tree in one of two
// layouts (dk_bvh.cu): 8 x float4 per 4-wide node with FP32 child boxes (x-min,
// x-max, y-min, y-max, z-min, z-max rows with one lane per child, the four
// child references, a spare row), or, with `wide8`, 5 x 16 bytes per 8-wide
// node with 8-bit quantised child boxes.
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
    uint64_t traversal_bytes;  // triangle slots + nodes, one block starting at `isect` (host bookkeeping)
    uint32_t light_count, env_count, env_tex_plus1, all_shadow_opaque;
    float env_intensity, env_rot_y, env_max_radiance;
    uint32_t env_guide_size;
    float env_rot_sin, env_rot_cos;  // sincosf(env_rot_y), evaluated once on the device
    uint32_t wide8;                  // traversal tree layout: 0 = 4-wide FP32, 1 = 8-wide quantised
    uint32_t watertight;             // triangle test: 0 = Moller-Trumbore over edges, 1 = watertight over vertices
    // Sparse distance volumes (GPUVolumeDescriptor with metadata.w == 1).
    const dk_volume_descriptor* volumes;
    const dk_volume_brick_descriptor* bricks;
    const dk_volume_brick_sample* brick_samples;
    const float* brick_dist;  // distance-only copy of brick_samples (FP32), or null
    const uint16_t* brick_dist16;  // the same as FP16 bits when every distance is a half value, or null
    const dk_volume_brick_grid* brick_grids;
    const uint32_t* brick_grid_indices;
    uint64_t brick_sample_count, brick_grid_index_count;
    uint32_t volume_count, brick_count, brick_grid_count, volume_all_opaque;
    // The reference's 13 SDF traversal counters (RenderSettings.collectsSDFTraversalStats), or null.
    unsigned long long* sdf_counters;
};
constexpr uint32_t kSdfCounterSlots = 13;

// GPURenderConstants (PathTrace.metal:143-182) for one batch of samples of
// one render.
struct DevParams {
    uint32_t width, height, max_bounces, transparent_background;
    uint32_t shows_env_bg, frame_seed, denoiser, pad0;
    float bg[3];
    float clamp;
    uint32_t tile_x, tile_y, tile_w, tile_h;
    uint32_t sample_begin, samples_in_batch, path_count, pad1;
    dk_camera cam, prev_cam;
};

struct alignas(32) D4 { double x, y, z, w; };

// Per-pixel accumulation of one render (a session or a serving job).
struct Accum {
    float4* sum;       // Kahan sum
    float4* comp;      // Kahan compensation
    D4* resolved;      // FP64 resolve of every completed 4096-sample block
    uint32_t* count;   // samples accumulated per pixel
    float4* aov;       // 6 planes: depth, normal, albedo, materialID, objectID, motion
};

// One render in a wave: a session's batch of samples over a tile, or one
// serving job's share of the wave.  Its paths are [path_begin, path_begin +
// P.path_count) of the wave (sample slice major, tile pixel minor) and its
// tile pixels [pixel_begin, pixel_begin + tile_w * tile_h) of the wave's AOV
// record.  Its materials are S.mats[mat_base, mat_base + mat_count): the
// shared geometry's material IDs index the job's own table.  After generation
// a path carries its job index in bits 8..31 of its flags.
// `opaque_mask` bit i: material i of the job's table blocks shadow rays
// (shadowOccluded, PathTrace.metal:4230-4241: not a cut-out, no
// transmission); material IDs from 32 up use the flag baked into the
// triangle slot.
struct DevJob {
    DevParams P;
    Accum A;
    uint32_t path_begin;
    uint32_t pixel_begin;
    uint32_t mat_base;
    uint32_t mat_count;
    uint32_t opaque_mask;
    uint32_t pad[3];
};

// SoA path state of one batch ("wave") of at most `cap` paths, shared by the
// `job_count` renders of `jobs` (ascending path_begin and pixel_begin).
struct Wave {
    float4* ray_o;     // origin
    float4* ray_d;     // direction
    float4* tp;        // throughput, w = previous BSDF pdf
    float4* rad;       // radiance, w = alpha
    uint2* rng;        // RNG state, flags (bit 0: primary hit found; bits 8..31: job index)
    float4* hit;       // t, triangle, u, v
    // NEE slots are indexed by the path's position in the shading order.
    float4* nee_o;     // 3 slots x cap: shadow origin, w = max distance
    float4* nee_d;     // 3 slots x cap: shadow direction, w = job index (bits)
    float4* nee_c;     // 3 slots x cap: unshadowed contribution, w = pdf divisor
    float4* nee_tp;    // throughput at NEE, w = slot mask | path index << 3 (bits)
    uint32_t* q[2];    // active path queues (ping-pong)
    uint32_t* qs;      // shading-order indices of paths with shadow queries
    uint32_t* qr;      // shadow rays: shading-order index << 2 | slot (3 x cap entries)
    uint32_t* qr2;     // shadow rays that need the layer walk (3 x cap entries)
    uint32_t* counts;  // [0], [1] queue lengths, [2] shadow paths, [3] shadow rays, [4] extend cursor,
                       // [5] shadow cursor, [6] layer-walk rays, [7] spare
    float4* aov;       // 4 planes of aov_stride tile pixels: primary-hit record of each job's last sample
    uint2* layer_hits;      // kRecLayers per shadow-ray slot: (t bits, triangle slot) of crossed non-opaque triangles
    uint32_t* layer_count;  // per shadow-ray slot: recorded layers, bit 31 = more than kRecLayers
    uint8_t* live;     // per path: 1 when it goes on to the next bounce (written by shading)
    uint32_t* scan;    // per block of kLiveBlock paths: live count, then its queue offset
    uint32_t* qsorted; // the active queue reordered by material (the shading order)
    uint32_t* keys;    // material key of each active-queue entry
    uint32_t* bins;    // kSortBins + 1 counters: key histogram, then bucket cursors
    const DevJob* jobs;
    uint32_t cap;
    uint32_t aov_stride;
    uint32_t job_count;
    uint32_t path_count;   // sum of the jobs' path counts
    uint32_t pixel_count;  // sum of the jobs' tile pixels
    uint32_t pad;
};

// Display encoding and PNG export (dk_image.cu).
cudaError_t encodeRgba8(const float4* px, uint32_t n, int kind, uint32_t* ws, uint32_t* out, cudaStream_t st);
int writePng(const char* path, const uint8_t* rgba, uint32_t w, uint32_t h);

// Host-side traversal BVH (dk_bvh.cu).
bool referenceSlots(const dk_scene* sc, std::vector<uint32_t>& slotOfTri, std::string& err);
// `width` 4 or 8 selects the node layout.
int buildSahTraversal(const dk_scene* sc, const std::vector<uint32_t>& slotOfTri, const std::vector<uint8_t>& opaque,
                      int width, std::vector<float4>& nodes, std::vector<float4>& isect, std::string& err);

cudaError_t launchGenerate(const DevScene& S, const Wave& W, int grid, cudaStream_t st);
cudaError_t launchExtend(const DevScene& S, const Wave& W, uint32_t sel, uint32_t bounce, int grid, int volumeGrid,
                         cudaStream_t st);
cudaError_t launchShade(const DevScene& S, const Wave& W, uint32_t bounce, uint32_t sel, int grid, cudaStream_t st);
cudaError_t launchShadow(const DevScene& S, const Wave& W, int grid, cudaStream_t st);
cudaError_t launchResolve(const Wave& W, int grid, cudaStream_t st);
cudaError_t launchAovPrimary(const DevScene& S, const Wave& W, int grid, cudaStream_t st);
// RenderQuality.preview / .interactive: one shading pass over the tile of `P`
// into the accumulation (overwritten) and its AOV planes.
cudaError_t launchPreview(const DevScene& S, const DevParams& P, const Accum& A, uint32_t matCount,
                          uint32_t opaqueMask, bool interactive, int grid, cudaStream_t st);
cudaError_t launchFinalize(const Wave& W, int grid, cudaStream_t st);
uint32_t bounceLaunches(const DevScene& S);
cudaError_t envRotation(float radians, float* sinCos /* device, 2 floats */, cudaStream_t st);
cudaError_t launchResolveBeauty(const Accum& A, uint32_t pixels, float4* out, int grid, cudaStream_t st);
cudaError_t buildEnvironmentTable(const float4* dPixels, uint32_t w, uint32_t h, float intensity, float maxR,
                                  double* dWeights, double* dPrefix, double* dBlockSums, float2* dOut, int grid,
                                  cudaStream_t st, double* hostTotal);

}  // namespace dk
