/*
 * denrim_cuda.h — C ABI of the GB300 (sm_103a) progressive path-tracing backend.
 *
 * This header is the drop-in seam for DenrimRendererKit's `final`-quality path
 * tracer (and the preview / interactive kernels of the same dispatch point).
 * The reference binds its GPU work in `RenderSession.init`
 * (Sources/DenrimRendererKit/Renderer/RenderSession.swift:292-579), which turns a
 * `RenderScene` into an `AccelerationBuild`
 * (Sources/DenrimRendererKit/Acceleration/AccelerationBuild.swift:4-48) and then
 * dispatches `pathTraceKernel`
 * (Sources/DenrimRendererKit/Resources/Shaders/PathTrace.metal:5167-5586) once per
 * sample from `RenderSession.encodeNextSample` (RenderSession.swift:891-1007).
 *
 * The functions below receive exactly the `AccelerationBuild` arrays as plain
 * old data with the byte layouts of Sources/DenrimRendererKit/Metal/GPUTypes.swift,
 * so a Swift `RenderSession` (or any other host) can hand its arrays over
 * unchanged.  Every function returns an `int` status (dk_status); the message of
 * the last failure on the calling thread is returned by dk_last_error_message().
 *
 * Threading: one session is single-threaded (the reference `RenderSession` is a
 * non-Sendable class); different sessions may be used from different threads.
 */
#ifndef DENRIM_CUDA_H
#define DENRIM_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------- */
/* Status codes.  1..5 map one-to-one onto `DenrimRendererError`             */
/* (Sources/DenrimRendererKit/Renderer/DenrimRenderer.swift:5-26).           */
/* ------------------------------------------------------------------------- */
typedef enum dk_status {
    DK_OK = 0,
    DK_ERROR_NO_DEVICE = 1,          /* noMetalDevice: no usable CUDA device          */
    DK_ERROR_MISSING_KERNEL = 2,     /* missingShaderFunction: kernel image absent    */
    DK_ERROR_INVALID_SCENE = 3,      /* invalidScene(reason)                          */
    DK_ERROR_COMMAND_FAILED = 4,     /* commandBufferFailed: a launch or copy failed  */
    DK_ERROR_EXPORT_FAILED = 5,      /* pngExportFailed                               */
    DK_ERROR_INVALID_ARGUMENT = 6,   /* null pointer, bad size or bad enum value      */
    DK_ERROR_OUT_OF_MEMORY = 7,      /* device allocation refused                     */
    DK_ERROR_DEVICE_TIMEOUT = 8      /* a bounded device-side wait gave up            */
} dk_status;

/* ------------------------------------------------------------------------- */
/* GPU struct ABI (GPUTypes.swift).  Sizes are checked by static asserts in  */
/* the library and by the Python ctypes mirror.                              */
/* ------------------------------------------------------------------------- */
typedef struct dk_float4 { float x, y, z, w; } dk_float4;
typedef struct dk_uint4 { uint32_t x, y, z, w; } dk_uint4;

/* GPUCamera, 80 B (GPUTypes.swift:4-10): origin.w = 1 for orthographic;
 * lens = {apertureRadius, focusDistance, 0, 0}. */
typedef struct dk_camera {
    dk_float4 origin;
    dk_float4 lower_left;
    dk_float4 horizontal;
    dk_float4 vertical;
    dk_float4 lens;
} dk_camera;

/* GPUTriangle, 192 B (GPUTypes.swift:12-28).  padding2 = light index + 1
 * (LightingGPUEncoding.swift:52) or 0 for a non-emissive triangle. */
typedef struct dk_triangle {
    dk_float4 v0, v1, v2;
    dk_float4 n0, n1, n2;
    dk_float4 uv0, uv1, uv2;
    dk_float4 tangent, bitangent;
    uint32_t material_id;
    uint32_t object_id;
    uint32_t primitive_id;
    uint32_t padding2;
} dk_triangle;

/* GPUMaterial, 17 x float4 = 272 B (GPUTypes.swift:30-48); the packing of the
 * user-facing fields is `Material.gpuMaterial` (Scene/Material.swift:222-284). */
typedef struct dk_material {
    dk_float4 base_color;              /* xyz base colour, w opacity                     */
    dk_float4 emission;                /* xyz emission*strength, w transmission          */
    dk_float4 parameters;              /* roughness, metallic, baseTex+1, normalMap+1    */
    dk_float4 parameters2;             /* specular, ior, clearcoat, clearcoatRoughness   */
    dk_float4 specular_color;          /* xyz tint, w clearcoat ior                      */
    dk_float4 sheen_color;             /* xyz tint, w sheen                              */
    dk_float4 transmission_color;      /* xyz tint, w thinWalled (0/1)                   */
    dk_float4 parameters3;             /* sheenRough, transRough, transIOR, anisotropy   */
    dk_float4 clearcoat_color;
    dk_float4 clearcoat_attenuation;   /* xyz colour, w thickness                        */
    dk_float4 transmission_absorption; /* xyz colour, w distance                         */
    dk_float4 thin_film;               /* strength, thickness nm, ior, 0                 */
    dk_float4 subsurface_color;        /* xyz colour, w subsurface                       */
    dk_float4 subsurface_radius;       /* xyz radius, w scale                            */
    dk_float4 subsurface_parameters;   /* anisotropy, 0, 0, 0                            */
    dk_float4 volume_scattering;       /* xyz colour, w scattering                       */
    dk_float4 volume_parameters;       /* distance, anisotropy, 0, 0                     */
} dk_material;

/* GPUAccelerationNode, 48 B (GPUTypes.swift:137-141, FlatBVH.swift:21-32):
 * metadata = {left, right, firstPrimitive, primitiveCount}; leaf iff count > 0. */
typedef struct dk_bvh_node {
    dk_float4 bounds_min;
    dk_float4 bounds_max;
    dk_uint4 metadata;
} dk_bvh_node;

/* GPUTextureDescriptor, 16 B: {pixelOffset, width, height, samplingMode}
 * (MaterialGPUEncoding.swift:26-33); samplingMode 0 nearest, 1 linear. */
typedef struct dk_texture_descriptor { dk_uint4 metadata; } dk_texture_descriptor;

/* GPULightRecord, 32 B (GPUTypes.swift:54-60). */
typedef struct dk_light_record {
    uint32_t triangle_index;
    uint32_t material_index;
    float area;
    float selection_cdf;
    dk_float4 normal;
} dk_light_record;

/* GPUEnvironmentSample, 8 B (GPUTypes.swift:62-64): {cdf, pdfSolidAngle}. */
typedef struct dk_environment_sample { float cdf; float pdf_solid_angle; } dk_environment_sample;

/* GPUVolumeDescriptor, 240 B (GPUTypes.swift:66-82).  Only sparse-brick
 * volumes (metadata.w == 1) are traced by this backend. */
typedef struct dk_volume_descriptor {
    dk_float4 world_bounds_min, world_bounds_max;
    dk_float4 local_bounds_min, local_bounds_max;
    dk_uint4 dimensions;
    dk_uint4 metadata;
    dk_uint4 material_program;
    dk_float4 world_to_local[4];
    dk_float4 normal_transform[4];
} dk_volume_descriptor;

/* GPUVolumeBrickSample, 16 B (GPUTypes.swift:95). */
typedef struct dk_volume_brick_sample {
    float distance;
    uint32_t material_a;
    uint32_t material_b;
    float material_blend;
} dk_volume_brick_sample;

/* GPUVolumeBrickDescriptor, 128 B (GPUTypes.swift:119-128). */
typedef struct dk_volume_brick_descriptor {
    dk_float4 world_bounds_min, world_bounds_max;
    dk_float4 local_bounds_min, local_bounds_max;
    dk_float4 sample_bounds_min, sample_bounds_max;
    dk_uint4 grid_origin_and_volume;
    dk_uint4 dimensions_and_sample_offset;
} dk_volume_brick_descriptor;

/* GPUVolumeBrickGrid, 64 B (GPUTypes.swift:130-135). */
typedef struct dk_volume_brick_grid {
    dk_uint4 dimensions_and_index_offset;
    dk_uint4 brick_size_and_volume;
    dk_uint4 macro_dimensions_and_index_offset;
    dk_uint4 macro_size_and_reserved;
} dk_volume_brick_grid;

/* ------------------------------------------------------------------------- */
/* The scene: the POD arrays of `AccelerationBuild` (AccelerationBuild.swift) */
/* plus the environment settings that `RenderSession` copies into            */
/* GPURenderConstants (RenderSession.swift:908-947).  The library copies     */
/* everything into device memory inside dk_session_create; the caller's      */
/* arrays may be freed as soon as it returns.                                */
/* ------------------------------------------------------------------------- */
typedef struct dk_scene {
    const dk_triangle* triangles;                 uint32_t triangle_count;
    const dk_material* materials;                 uint32_t material_count;
    const dk_bvh_node* nodes;                     uint32_t node_count;
    const uint32_t* primitive_indices;            uint32_t primitive_index_count;
    const dk_texture_descriptor* texture_descriptors; uint32_t texture_descriptor_count;
    const dk_float4* texture_pixels;              uint64_t texture_pixel_count;
    const dk_light_record* lights;                uint32_t light_count;
    const dk_environment_sample* environment_samples; uint32_t environment_sample_count;
    uint32_t environment_texture_index_plus_one;
    float environment_intensity;                  /* Environment.intensity   */
    float environment_rotation_y;                 /* Environment.rotationY   */
    float environment_max_radiance;               /* Environment.maxRadiance */
    /* Sparse distance-volume bricks (SparseVolumeGPUEncoding.swift:9-299). */
    const dk_volume_descriptor* volumes;          uint32_t volume_count;
    const dk_volume_brick_descriptor* volume_bricks; uint32_t volume_brick_count;
    const dk_volume_brick_sample* volume_brick_samples; uint64_t volume_brick_sample_count;
    const dk_volume_brick_grid* volume_brick_grids; uint32_t volume_brick_grid_count;
    const uint32_t* volume_brick_grid_indices;    uint64_t volume_brick_grid_index_count;
} dk_scene;

/* RenderQuality (RenderSettings.swift:5-26), the kernel a session runs
 * (DenrimRenderer.primaryPipeline, DenrimRenderer.swift:197-214): FINAL the
 * path tracer (pathTraceKernel), PREVIEW the flat preview (flatPreviewKernel,
 * PathTrace.metal:4728-4868), INTERACTIVE the direct-light material preview
 * (interactiveMaterialKernel, :4870-5165).  The two previews overwrite the
 * image on every sample. */
enum { DK_QUALITY_PREVIEW = 0, DK_QUALITY_INTERACTIVE = 1, DK_QUALITY_FINAL = 2 };

/* RenderSettings (RenderSettings.swift:29-116) plus the two cameras. */
typedef struct dk_settings {
    uint32_t width;
    uint32_t height;
    uint32_t max_bounces;                 /* clamped to >= 1 like RenderSession.swift:915 */
    uint32_t quality;                     /* DK_QUALITY_*                                  */
    uint32_t transparent_background;
    uint32_t shows_environment_background;
    float background_color[3];
    uint32_t sample_radiance_clamp_set;   /* 0: inherit RenderQuality default (64 final)  */
    float sample_radiance_clamp;          /* used when _set != 0; 0 disables the clamp     */
    uint32_t frame_seed;                  /* reference hard-wires 0x1234ABCD               */
    uint32_t denoiser_enabled;            /* 1: trace the unjittered AOV ray (PathTrace.metal:5530-5557) */
    uint32_t collects_traversal_stats;
    dk_camera camera;
    dk_camera previous_camera;
    uint32_t max_samples_per_launch;      /* 0: the library picks; caps one wavefront batch */
    uint32_t triangle_test;               /* DK_TRIANGLE_TEST_*; 0 (the reference's test) by default */
} dk_settings;

/* Ray-triangle test of a session.  MOLLER_TRUMBORE is the reference's
 * intersectTriangle (PathTrace.metal:1801-1852) and the only mode with
 * bit-exact parity against it.  WATERTIGHT is the shear-and-edge-function test
 * of Woop, Benthin and Wald (JCGT 2013): no ray slips through a shared edge or
 * vertex; hits near edges may differ from the reference's in the last bits. */
#define DK_TRIANGLE_TEST_MOLLER_TRUMBORE 0u
#define DK_TRIANGLE_TEST_WATERTIGHT 1u

/* RenderOutput (Renderer/RenderOutput.swift:4-25). */
typedef enum dk_output {
    DK_OUTPUT_BEAUTY = 0,
    DK_OUTPUT_DEPTH = 1,
    DK_OUTPUT_NORMAL = 2,
    DK_OUTPUT_ALBEDO = 3,
    DK_OUTPUT_MATERIAL_ID = 4,
    DK_OUTPUT_OBJECT_ID = 5,
    DK_OUTPUT_MOTION_VECTOR = 6
} dk_output;

/* Per-session counters.  The first 13 are the reference's SDF traversal
 * counters in its slot order (PathTrace.metal:191-203); the rest time and
 * count this backend's own work. */
typedef struct dk_stats {
    uint64_t sdf_counters[13];
    uint64_t paths_traced;                /* pixel-samples completed since create       */
    uint64_t rays_extended;               /* closest-hit queries issued                  */
    uint64_t shadow_rays;                 /* shadow queries issued                       */
    uint64_t kernel_launches;             /* kernels launched since create               */
    double last_render_ms;                /* device time of the last dk_session_render  */
    double last_extend_ms;                /* of which: closest-hit (extend) kernels      */
    double last_shade_ms;                 /* of which: shading kernels                   */
    double last_shadow_ms;                /* of which: shadow kernels                    */
    double last_other_ms;                 /* of which: generate / accumulate / AOV       */
    uint64_t last_launches;               /* kernels launched by the last render call    */
    uint64_t device_bytes;                /* device memory held by the session           */
} dk_stats;

typedef struct dk_session dk_session;

/* ------------------------------------------------------------------------- */
/* Device and session API.                                                    */
/* ------------------------------------------------------------------------- */

/* Selects and initialises a CUDA device (DenrimRenderer.init,
 * DenrimRenderer.swift:52-70).  Returns DK_ERROR_NO_DEVICE when none exists. */
int dk_device_open(int device_ordinal);

/* Number of CUDA devices visible to the process (0 without a GPU). */
int dk_device_count(int* out_count);

/* DenrimRenderer.makeSession(scene:settings:accelerationMode:)
 * (DenrimRenderer.swift:253-292) + RenderSession.init (RenderSession.swift:292-579).
 * Validation follows RenderSession.swift:304-327: non-positive size, no
 * geometry or no materials fail with DK_ERROR_INVALID_SCENE. */
int dk_session_create(const dk_scene* scene, const dk_settings* settings, dk_session** out_session);

/* RenderSession.render(samples:) (RenderSession.swift:1010-1017): adds
 * `samples` progressive samples over the full frame.  On failure the sample
 * count is left unchanged (RenderSession.swift:844-847). */
int dk_session_render(dk_session* session, uint32_t samples);

/* RenderSession.renderNextTile(_:completesSample:) (RenderSession.swift:875-889):
 * one sample over a tile; the sample index advances only when
 * completes_sample != 0. */
int dk_session_render_tile(dk_session* session, uint32_t x, uint32_t y, uint32_t width,
                           uint32_t height, int completes_sample);

/* RenderSession.updateCamera(_:previousCamera:) (RenderSession.swift:595-608).
 * `previous` may be NULL: the camera active before the update is used.
 * Restarts accumulation. */
int dk_session_update_camera(dk_session* session, const dk_camera* camera, const dk_camera* previous);

/* RenderSession.resetAccumulation() (RenderSession.swift:582-588). */
int dk_session_reset(dk_session* session);

/* RenderSession.pixels(for:) (RenderSession.swift:1037-1039): copies the
 * output as RGBA32F into `rgba` (pixel_count = width*height pixels). */
int dk_session_read_output(dk_session* session, int output, float* rgba, size_t pixel_count);

/* RenderSession.texture(for:) (RenderSession.swift:1072-1094), the
 * device-resident output the reference hands to its viewport and denoiser:
 * copies the output as RGBA32F into caller-owned DEVICE memory `device_rgba`
 * (pixel_count = width*height pixels, 16-byte aligned), with no host
 * round trip.  The copy is ordered before work queued afterwards on `stream`
 * (a cudaStream_t; NULL: the call returns when the copy is complete). */
int dk_session_copy_output(dk_session* session, int output, void* device_rgba, size_t pixel_count, void* stream);

/* PNGWriter.visualizedRGBA8Pixels (Image/PNGWriter.swift:35-53) on the device:
 * the output as the reference's PNG export shows it (beauty tonemapped, depth
 * normalised to its range, IDs hashed to colours, ...), 8-bit RGBA, row major,
 * width*height*4 bytes into host `rgba`. */
int dk_session_read_rgba8(dk_session* session, int output, uint8_t* rgba, size_t bytes);

/* RenderSession.writePNG(output:to:) (RenderSession.swift:1026-1034): the
 * output encoded as above, written as an 8-bit RGBA PNG file at `path`.
 * DK_ERROR_EXPORT_FAILED when the file cannot be written. */
int dk_session_write_png(dk_session* session, int output, const char* path);

/* The same encoding of caller-owned device pixels: `pixels` RGBA32F (16-byte
 * aligned, width*height), `rgba` device bytes (width*height*4, 4-byte
 * aligned), `workspace` DK_ENCODE_WORKSPACE_BYTES of device memory; launched
 * on `stream` (a cudaStream_t, may be null), not synchronised. */
#define DK_ENCODE_WORKSPACE_BYTES 16
int dk_encode_rgba8(const float* pixels, uint32_t width, uint32_t height, int output, uint8_t* rgba,
                    void* workspace, void* stream);

/* PNGWriter.write (PNGWriter.swift:55-70): host 8-bit RGBA bytes as a PNG file. */
int dk_write_png(const char* path, const uint8_t* rgba, uint32_t width, uint32_t height);

/* RenderSession.sampleCount. */
int dk_session_sample_count(const dk_session* session, uint32_t* out_count);

/* RenderSession.sdfTraversalStats() (RenderSession.swift:808-831) plus timing.
 * `sdf_counters` holds the reference's 13 counter slots (PathTrace.metal:191-203)
 * when the session was created with `collects_traversal_stats`, else zeros. */
int dk_session_stats(const dk_session* session, dk_stats* out_stats);
/* RenderSession.resetSDFTraversalStats() (RenderSession.swift:611-614): zeroes the SDF traversal counters. */
int dk_session_reset_sdf_stats(dk_session* session);

/* Releases every device buffer of the session. */
int dk_session_destroy(dk_session* session);

/* Message of the last failure on this thread ("" when none). */
const char* dk_last_error_message(void);

/* ------------------------------------------------------------------------- */
/* Scene-compile helpers: GB300 restatements of the Swift host builders a    */
/* caller without them needs in order to fill dk_scene.                      */
/* ------------------------------------------------------------------------- */

/* BVHBuilder.build(triangles:) + BVHFlattener.flatten
 * (Acceleration/BVHBuilder.swift:7-92, FlatBVH.swift:13-32): median split on
 * the largest centroid axis, stable ordering, pre-order node numbering.
 * `nodes_out` must hold 2*triangle_count nodes, `primitive_indices_out`
 * triangle_count entries; *node_count receives the node count. */
int dk_build_bvh(const dk_triangle* triangles, uint32_t triangle_count, uint32_t max_leaf_primitives,
                 dk_bvh_node* nodes_out, uint32_t* node_count, uint32_t* primitive_indices_out);

/* LinearTriangleAccelerationBackend.lightRecordsAndTaggedTriangles
 * (Acceleration/LightingGPUEncoding.swift:5-64): writes padding2 = light+1
 * into `triangles` in place and fills `lights_out` (capacity triangle_count).
 * *light_count receives the number of emissive-triangle lights. */
int dk_build_lights(dk_triangle* triangles, uint32_t triangle_count, const dk_material* materials,
                    uint32_t material_count, dk_light_record* lights_out, uint32_t* light_count);

/* LinearTriangleAccelerationBackend.environmentSamples
 * (Acceleration/LightingGPUEncoding.swift:66-119), computed on the GPU with an
 * FP64 prefix sum and stored as FP32.  `out` holds width*height entries;
 * *out_count is 0 when the map carries no energy (the reference's empty case). */
int dk_build_environment_samples(const dk_float4* pixels, uint32_t width, uint32_t height, float intensity,
                                 float max_radiance, dk_environment_sample* out, uint32_t* out_count);

/* Sparse distance volume for models of sphere primitives, the input of the
 * sparse-brick path (GPUVolumeDescriptor metadata.w == 1).  Restates
 * DistanceVolumeBuilder.buildSparse (Scene/SDFModel.swift:255-355, 2-voxel
 * stored overlap, narrow-band brick selection), gpuVolumeBricks
 * (Acceleration/SparseVolumeGPUEncoding.swift:9-299, brick grid + 4^3 macro
 * occupancy) and appendSparseVolumeDescriptor (VolumeGPUEncoding.swift:184-243)
 * for an identity instance transform.  The primitives are combined in order by
 * union with the polynomial smooth minimum of `smooth_union_radius`. */
typedef struct dk_sdf_sphere {
    float center[3];
    float radius;
    uint32_t material;
    float smooth_union_radius;
} dk_sdf_sphere;

typedef struct dk_sparse_volume_settings {
    uint32_t resolution[3];   /* samples per axis of the virtual grid        */
    float bounds_min[3];
    float bounds_max[3];
    uint32_t brick_size[3];   /* core brick size in samples                   */
    float narrow_band;        /* keep bricks with min <= band && max >= -band */
    uint32_t volume_material; /* the volume's fallback material               */
    uint32_t object_id;
    uint32_t primitive_id;
    uint32_t fp16_distances;  /* 1: store every sample distance rounded to half precision (the
                               * packed records keep the rounded value as FP32; the march then
                               * reads 2 bytes a sample).  No counterpart in the reference. */
} dk_sparse_volume_settings;

typedef struct dk_sparse_volume dk_sparse_volume;

int dk_build_sparse_sphere_volume(const dk_sdf_sphere* spheres, uint32_t sphere_count,
                                  const dk_sparse_volume_settings* settings, dk_sparse_volume** out_volume);

/* The same volume baked on the current CUDA device (DistanceFieldBaker's
 * sparse GPU path, Scene/DistanceFieldBaker.swift:700-966 with
 * SDFBake.metal:1056-1200: classify bricks, sample the kept ones), bit-identical
 * to dk_build_sparse_sphere_volume; the arrays are returned in host memory. */
int dk_bake_sparse_sphere_volume(const dk_sdf_sphere* spheres, uint32_t sphere_count,
                                 const dk_sparse_volume_settings* settings, dk_sparse_volume** out_volume);

/* Points the volume fields of `scene` at the built arrays (owned by the volume). */
int dk_sparse_volume_view(const dk_sparse_volume* volume, dk_scene* scene);

int dk_sparse_volume_destroy(dk_sparse_volume* volume);

/* Allocation-free variant of dk_build_environment_samples.  It has no
 * counterpart in the reference.  It serves callers that cannot let the library
 * call cudaMalloc: applications that give the renderer only device memory from
 * their own arena or pool, and real-time frame loops that must not allocate.
 * The caller passes DEVICE pointers: `device_pixels` (width*height float4
 * texels, 16-byte aligned) and `device_out` (width*height entries, 8-byte
 * aligned); host or misaligned pointers fail with DK_ERROR_INVALID_ARGUMENT.
 * The FP64 prefix-sum scratch
 * is one static __device__ array sized for DK_ENV_NOALLOC_MAX_TEXELS texels
 * (2048 x 1024, 16 MiB), held by every GPU that loads this library until the
 * process exits; larger maps fail with DK_ERROR_INVALID_ARGUMENT.  The first
 * call on a device looks up the array's device address (make that first call
 * before any stream capture).  All calls share the one array: calls that
 * overlap on the GPU (other threads, other streams) race.  Works on `stream`
 * (NULL: the default stream) and returns after the table is complete (it
 * reads the table's total back to the host, so a call on a stream that is
 * being captured fails with DK_ERROR_INVALID_ARGUMENT);
 * *out_count is width*height, or 0 for a map without energy.  Allocates
 * nothing: no cudaMalloc, no cudaFree, no allocating library routine. */
#define DK_ENV_NOALLOC_MAX_TEXELS (2048u * 1024u)
int dk_build_environment_samples_noalloc(const dk_float4* device_pixels, uint32_t width, uint32_t height,
                                         float intensity, float max_radiance, dk_environment_sample* device_out,
                                         uint32_t* out_count, void* stream);

/* Library version string. */
const char* dk_version(void);

/* Measured read bandwidth of the current device in GB/s: `passes` sweeps of
 * 16-byte loads over a `bytes` buffer (>= 1 MiB) after one warm-up sweep,
 * timed with CUDA events on `stream`.  A buffer well inside L2 (e.g. 64 MiB of
 * the 129 MB) measures L2, one far larger HBM.  Allocates and frees the
 * buffer; blocks until done.  Measurement only (the traversal stages'
 * rooflines are stated against it); no counterpart in the reference. */
int dk_probe_bandwidth(uint64_t bytes, uint32_t passes, double* out_gbs, void* stream);

/* ------------------------------------------------------------------------- */
/* Denoising.                                                                 */
/* ------------------------------------------------------------------------- */

/* DenoiseSettings for the simple spatial denoiser
 * (Sources/DenrimRendererKit/Denoising/Denoiser.swift:20-77). */
typedef struct dk_spatial_denoise_settings {
    uint32_t radius;        /* clamped to 1..2 */
    float normal_sigma;
    float depth_sigma;
    float albedo_sigma;
    float color_sigma;
    uint32_t iterations;    /* a-trous passes, clamped to 1..5; step width 1 << pass */
} dk_spatial_denoise_settings;

/* Replaces SimpleSpatialDenoiser.encode (Denoiser.swift:103-160) running
 * simpleSpatialDenoiseKernel (Denoise.metal:39-115).  All image pointers are
 * DEVICE RGBA32F planes of width*height texels (beauty, depth, encoded normal,
 * albedo AOVs as dk_session_read_output lays them out); `scratch` holds two
 * planes (may be null for one pass); `stream` is a cudaStream_t or null.
 * Asynchronous on `stream`. */
int dk_denoise_spatial(const float* beauty, const float* depth, const float* normal, const float* albedo,
                       float* out, float* scratch, uint32_t width, uint32_t height,
                       const dk_spatial_denoise_settings* settings, void* stream);

/* The sums behind the learned denoiser's per-image error estimate, for
 * `images` images of `pixels` RGBA32F pixels each (DEVICE pointers, images
 * back to back): two independent half-sample renders A and B, the full render
 * F of the same samples, and the three denoised images.  `terms` (DEVICE,
 * images x 5 doubles, overwritten) receives per image the sums over pixels and
 * RGB of (dA - dB)^2, (A - B)^2, (F - dF)^2, dF and F -- of the linear values
 * (`display` 0) or of the displayed ones (`display` 1: the reference's PNG
 * tone curve, PNGWriter.swift:182-188, before quantisation).  Asynchronous on
 * `stream`.  No counterpart in the reference (its denoisers carry no error
 * estimate); it drives the fallback to more samples of the serving loop. */
int dk_denoise_error_terms(const float* half_a, const float* half_b, const float* full, const float* denoised_a,
                           const float* denoised_b, const float* denoised_full, uint32_t pixels, uint32_t images,
                           uint32_t display, double* terms, void* stream);

/* out = (1 - t) a + t b over `texels` RGBA32F texels (DEVICE pointers; `out`
 * may alias `a` or `b`): the full render of two independent renders of n_a and
 * n_b samples with t = n_b / (n_a + n_b).  Asynchronous on `stream`. */
int dk_average_planes(const float* a, const float* b, float* out, size_t texels, float t, void* stream);

/* DenoiseSettings.appleSVGF (Denoiser.swift:67-76) -- AppleSVGFDenoiser
 * (Denoiser.swift:167-300) -- as spatiotemporal variance-guided filtering
 * (the published SVGF algorithm; the reference's implementation is Apple's
 * closed MPSSVGFDenoiser) with the parameters its configure(settings:) sets:
 * a-trous iterations clamp(iterations, 1, 5), filter and variance radius
 * clamp(radius, 1, 4), depth weight max(depth_sigma, 1e-4), normal weight
 * clamp(24 / normal_sigma, 1, 512), luminance weight max(color_sigma, 1e-4),
 * moving-average factor 0.2.  One object per image size holds the temporal
 * history; dk_svgf_reset is clearTemporalHistory.  dk_svgf_denoise takes
 * DEVICE RGBA32F planes (beauty, depth, encoded normal and motion-vector AOVs
 * as dk_session_copy_output lays them out) and writes `out`; asynchronous on
 * `stream`. */
typedef struct dk_svgf dk_svgf;
int dk_svgf_create(uint32_t width, uint32_t height, dk_svgf** out_svgf);
int dk_svgf_reset(dk_svgf* svgf);
int dk_svgf_denoise(dk_svgf* svgf, const float* beauty, const float* depth, const float* normal, const float* motion,
                    float* out, const dk_spatial_denoise_settings* settings, void* stream);
/* The filter state after the last dk_svgf_denoise, copied to device memory:
 * 0 history colour, 1 (luminance mean, mean square, history length, 0),
 * 2 packed (depth, signed normal). */
int dk_svgf_read_state(dk_svgf* svgf, int which, float* device_rgba, size_t pixel_count, void* stream);
int dk_svgf_destroy(dk_svgf* svgf);
/* packSVGFDepthNormalKernel (Denoise.metal:117-136) and copySVGFOutputKernel
 * (Denoise.metal:138-154) on their own, over device RGBA32F planes. */
int dk_svgf_pack_depth_normal(const float* depth, const float* normal, float* depth_normal, uint32_t width,
                              uint32_t height, void* stream);
int dk_svgf_copy_output(const float* denoised, const float* original, float* out, uint32_t width, uint32_t height,
                        void* stream);

/* Learned denoiser building blocks (no counterpart in the reference, whose
 * denoisers are the spatial filter above and Apple's SVGF).  Tensors are
 * DEVICE NHWC bf16 (raw 16-bit storage) with channel counts that are
 * multiples of 16; `ld*` is the channel stride of a pixel (a tensor may be a
 * channel slice of a wider buffer) and `*_off` a channel offset.  All calls
 * are asynchronous on `stream` (a cudaStream_t or null). */

/* 3x3 convolution, stride 1, zero padding 1, FP32 accumulation on the tensor
 * cores: out[p][co_off + co] (+)= act(bias[co] + sum in[p + tap][ci] *
 * weight[co][tap][ci]); act 0 = identity, 1 = ReLU; bias may be null.  With
 * the tap-flipped transposed weights (dk_unet_adam / dk_unet_weights_to_bf16
 * `wflip`) it computes the input gradient. */
int dk_unet_conv3x3(const void* in, uint32_t n, uint32_t h, uint32_t w, uint32_t cin, uint32_t ldi,
                    const void* weight, const float* bias, uint32_t cout, void* out, uint32_t ldo, uint32_t co_off,
                    int act, int accumulate, void* stream);
/* Weight gradient: dweight[co][tap][ci] += sum_p dout[p][co] * in[p + tap][ci] (FP32). */
int dk_unet_conv3x3_wgrad(const void* in, uint32_t ldi, const void* dout, uint32_t ldd, uint32_t n, uint32_t h,
                          uint32_t w, uint32_t cin, uint32_t cout, float* dweight, void* stream);
/* dpre = dout where out > 0. */
int dk_unet_relu_backward(const void* out, uint32_t ldo, const void* dout, uint32_t ldd, void* dpre, uint32_t ldp,
                          uint32_t c, uint32_t pixels, void* stream);
/* dbias[c] += sum_p dpre[p][c] (c <= 256). */
int dk_unet_bias_grad(const void* dpre, uint32_t ld, uint32_t c, uint32_t pixels, float* dbias, void* stream);
/* dk_unet_conv3x3 (no accumulation) followed by dk_unet_avgpool2 of the
 * channels it wrote: pool[q][c] (channel stride pool_ld, offset 0) = the 2x2
 * average of out's channels co_off .. co_off + cout; h and w even.  The same
 * bits as the two calls; where the convolution's rows leave by tensor stores
 * (16, 32 or 64 output channels, at most 128 input channels, w >= 128) its
 * epilogue averages the row pairs it has staged, so the output is not read back. */
int dk_unet_conv3x3_avgpool2(const void* in, uint32_t n, uint32_t h, uint32_t w, uint32_t cin, uint32_t ldi,
                             const void* weight, const float* bias, uint32_t cout, void* out, uint32_t ldo,
                             uint32_t co_off, int act, void* pool, uint32_t pool_ld, void* stream);
/* 2x2 average pooling of an (h, w) tensor, and its gradient. */
int dk_unet_avgpool2(const void* in, uint32_t ldi, void* out, uint32_t ldo, uint32_t co_off, uint32_t c, uint32_t n,
                     uint32_t h, uint32_t w, void* stream);
int dk_unet_avgpool2_backward(const void* dout, uint32_t ldd, void* din, uint32_t ldi, uint32_t c, uint32_t n,
                              uint32_t h, uint32_t w, int accumulate, void* stream);
/* Nearest 2x upsampling of an (h, w) tensor, and its gradient. */
int dk_unet_upsample2(const void* in, uint32_t ldi, void* out, uint32_t ldo, uint32_t co_off, uint32_t c, uint32_t n,
                      uint32_t h, uint32_t w, void* stream);
int dk_unet_upsample2_backward(const void* dout, uint32_t ldd, uint32_t ci_off, void* din, uint32_t ldi, uint32_t c,
                               uint32_t n, uint32_t h, uint32_t w, void* stream);
int dk_unet_copy_channels(const void* src, uint32_t lds, uint32_t s_off, void* dst, uint32_t ldd, uint32_t d_off,
                          uint32_t c, uint32_t pixels, int accumulate, void* stream);
/* 16-channel network input of batch item `batch_index` from an (h, w) window at
 * (x0, y0) of the RGBA32F AOV planes: log(1 + beauty), albedo, normal in
 * [-1, 1], depth / (1 + depth), zeros. */
int dk_unet_pack_input(const float* beauty, const float* albedo, const float* normal, const float* depth,
                       uint32_t image_width, uint32_t image_height, uint32_t x0, uint32_t y0, void* out, uint32_t h,
                       uint32_t w, uint32_t batch_index, void* stream);
/* L1 loss between the prediction's first 3 channels (log space) and
 * log(1 + target) (RGBA32F); loss (+)= mean, grad = its gradient. */
int dk_unet_l1_loss(const void* pred, uint32_t ldp, const float* target, uint32_t pixels, void* grad, uint32_t ldg,
                    float* loss, void* stream);
/* Prediction (log space) to an RGBA32F image window; alpha from alpha_src. */
int dk_unet_unpack_output(const void* pred, uint32_t ldp, uint32_t h, uint32_t w, const float* alpha_src,
                          uint32_t image_width, uint32_t image_height, uint32_t x0, uint32_t y0, float* out,
                          void* stream);
/* The same two with the prediction a residual over the network input `base`
 * (whose first 3 channels are log(1 + noisy beauty)): output = base + pred in
 * log space, summed in FP32, so a converged pixel (a visible light) keeps its
 * value to the residual's precision instead of the activations'. */
int dk_unet_l1_loss_residual(const void* pred, uint32_t ldp, const void* base, uint32_t ldb, const float* target,
                             uint32_t pixels, void* grad, uint32_t ldg, float* loss, void* stream);
int dk_unet_unpack_output_residual(const void* pred, uint32_t ldp, const void* base, uint32_t ldb, uint32_t h,
                                   uint32_t w, const float* alpha_src, uint32_t image_width, uint32_t image_height,
                                   uint32_t x0, uint32_t y0, float* out, void* stream);
/* Adam step on FP32 master weights; refreshes the bf16 copy and (3x3 layers,
 * wflip non-null) the tap-flipped transposed copy [cin][9][cout]. */
int dk_unet_adam(float* weights, const float* grad, float* m, float* v, uint32_t count, float lr, float beta1,
                 float beta2, float eps, uint32_t step, void* wbf16, void* wflip, uint32_t cout, uint32_t cin,
                 void* stream);
int dk_unet_weights_to_bf16(const float* weights, uint32_t count, void* wbf16, void* wflip, uint32_t cout,
                            uint32_t cin, void* stream);
/* Selects the convolution kernel (Cout <= 256 for the tcgen05 ones): 3
 * (default) the halo-row TMA + tcgen05 kernel for images at least 128 pixels
 * wide whose weights and input rows fit one CTA's shared memory, else 2;
 * 2 persistent per-tap TMA + tcgen05 with warp roles, 1 cp.async + tcgen05,
 * 0 mma.sync; the alternatives are kept for comparison. */
int dk_unet_set_conv_path(int path);
/* Reads and clears the denoiser kernels' error flag (non-zero: a bounded wait
 * for the tensor cores or a copy timed out and the affected tiles were not
 * written; 1, 2, 3 name the cp.async, per-tap TMA and halo-row kernels). */
int dk_unet_error(int* out_error);

/* ------------------------------------------------------------------------- */
/* Serving: a persistent request loop over one resident scene.                */
/* No counterpart in the reference: its RenderSession (RenderSession.swift)  */
/* renders one scene per session, one dispatch per sample.  A server keeps   */
/* the scene (triangles, BVH, textures, HDRI table) resident and renders     */
/* jobs -- each with its own settings, camera, sample count and material     */
/* table over the shared geometry -- by packing the paths of every admitted  */
/* job into one shared wavefront per wave.  Jobs are admitted first-in       */
/* first-out while their accumulation buffers fit the HBM budget; a job      */
/* admitted while others run joins the next wave.  A job's result equals the */
/* result of a session over the same scene with the job's materials and     */
/* settings, bit for bit.                                                    */
/* ------------------------------------------------------------------------- */
typedef struct dk_server dk_server;

typedef struct dk_server_config {
    uint64_t hbm_budget_bytes;     /* admission budget for per-job buffers; 0: 64 GiB            */
    uint32_t wave_paths;           /* path capacity of the shared wave; 0: 2^24                  */
    uint32_t max_jobs_per_wave;    /* 0: 512                                                     */
    uint32_t max_resident_jobs;    /* admitted and not yet released; 0: 4096                     */
    uint32_t samples_per_wave;     /* samples one job advances per wave at most; 0: 64           */
    uint32_t policy;               /* wave packing after the oldest running job: 0 admission      */
                                   /* order, 1 fewest remaining paths first                       */
    uint32_t reserved;
} dk_server_config;

/* One render request.  `materials` replaces the scene's material table for
 * this job (same count); it may change any material's parameters except
 * emission (the light list is the scene's) and, for material IDs from 32 up,
 * whether the material blocks shadow rays. */
typedef struct dk_job_desc {
    dk_settings settings;
    uint32_t samples;
    uint32_t material_count;
    const dk_material* materials;
    uint32_t scene;                /* resident scene: 0 the create-time one, else dk_server_add_scene's */
    uint32_t reserved;
} dk_job_desc;

enum { DK_JOB_QUEUED = 0, DK_JOB_RUNNING = 1, DK_JOB_DONE = 2, DK_JOB_RELEASED = 3 };

typedef struct dk_job_status {
    uint64_t job_id;
    uint32_t state;                /* DK_JOB_*                                                   */
    uint32_t samples_done;
    uint32_t samples;
    uint32_t waves;                /* waves the job took part in                                 */
    double submit_ms;              /* server clock (ms since dk_server_create)                   */
    double admit_ms;
    double finish_ms;
} dk_job_status;

typedef struct dk_server_stats {
    uint64_t jobs_submitted, jobs_done, jobs_queued, jobs_running;
    uint64_t waves, paths_traced, kernel_launches;
    uint64_t budget_used_bytes, budget_peak_bytes, device_bytes;
    double busy_ms;                /* device time of all waves                                   */
    double max_jobs_in_wave, mean_jobs_in_wave;
} dk_server_stats;

/* Uploads `scene` once and prepares the shared wave. */
int dk_server_create(const dk_scene* scene, const dk_server_config* config, dk_server** out_server);
/* Makes another scene resident in the server (its BVH, textures, lights and
 * HDRI table uploaded once, with its own wavefront of `wave_paths` paths and
 * stream); jobs name it by the returned index.  Every step runs one packed
 * wave per scene with work, the scenes' waves overlapping on the device.  No
 * counterpart in the reference, whose RenderSession holds one scene. */
int dk_server_add_scene(dk_server* server, const dk_scene* scene, uint32_t* out_scene);
/* Queues a job; validation errors are returned here (DK_ERROR_INVALID_*). */
int dk_server_submit(dk_server* server, const dk_job_desc* job, uint64_t* out_job_id);
/* Admits queued jobs and runs one wave on the calling thread; `out_jobs` (may
 * be null) receives the number of jobs in the wave (0: nothing to do). */
int dk_server_step(dk_server* server, uint32_t* out_jobs);
/* Runs waves on a background thread until dk_server_stop / destroy. */
int dk_server_start(dk_server* server);
int dk_server_stop(dk_server* server);
/* Blocks until the job is done (or `timeout_ms` passes: DK_ERROR_DEVICE_TIMEOUT). */
int dk_server_wait(dk_server* server, uint64_t job_id, uint32_t timeout_ms);
int dk_server_job_status(dk_server* server, uint64_t job_id, dk_job_status* out_status);
/* Reads a finished job's output (as dk_session_read_output). */
int dk_server_read_output(dk_server* server, uint64_t job_id, int output, float* rgba, size_t pixel_count);
/* Copies a finished job's output into caller-owned device memory (as
 * dk_session_copy_output): the hand-off of a batch of served images to a
 * denoiser without a host round trip. */
int dk_server_copy_output(dk_server* server, uint64_t job_id, int output, void* device_rgba, size_t pixel_count,
                          void* stream);
/* The same for `count` finished jobs of one size in one call: job i's output
 * goes to device_rgba + i * stride_bytes (0: pixel_count * 16, packed). */
int dk_server_copy_outputs(dk_server* server, const uint64_t* job_ids, size_t count, int output, void* device_rgba,
                           size_t pixel_count, size_t stride_bytes, void* stream);
/* Frees a finished job's buffers (its budget returns to admission). */
int dk_server_release(dk_server* server, uint64_t job_id);
int dk_server_get_stats(dk_server* server, dk_server_stats* out_stats);
int dk_server_destroy(dk_server* server);

#ifdef __cplusplus
}
#endif

#endif /* DENRIM_CUDA_H */
