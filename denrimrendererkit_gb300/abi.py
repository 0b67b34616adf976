"""ctypes / numpy mirrors of the C ABI in include/denrim_cuda.h.

The numpy dtypes give the byte layouts of the reference's GPU structs
(Sources/DenrimRendererKit/Metal/GPUTypes.swift), so scene arrays built here
can be handed to the library (and to the oracle) without copies.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

F4 = (np.float32, (4,))
U4 = (np.uint32, (4,))

# GPUTriangle, 192 B (GPUTypes.swift:12-28)
TRIANGLE_DTYPE = np.dtype([
    ("v0", F4), ("v1", F4), ("v2", F4),
    ("n0", F4), ("n1", F4), ("n2", F4),
    ("uv0", F4), ("uv1", F4), ("uv2", F4),
    ("tangent", F4), ("bitangent", F4),
    ("material_id", np.uint32), ("object_id", np.uint32),
    ("primitive_id", np.uint32), ("padding2", np.uint32),
])
# GPUMaterial, 17 x float4 = 272 B (GPUTypes.swift:30-48)
MATERIAL_FIELDS = (
    "base_color", "emission", "parameters", "parameters2", "specular_color", "sheen_color",
    "transmission_color", "parameters3", "clearcoat_color", "clearcoat_attenuation",
    "transmission_absorption", "thin_film", "subsurface_color", "subsurface_radius",
    "subsurface_parameters", "volume_scattering", "volume_parameters",
)
MATERIAL_DTYPE = np.dtype([(name, F4) for name in MATERIAL_FIELDS])
# GPUAccelerationNode, 48 B (GPUTypes.swift:137-141)
NODE_DTYPE = np.dtype([("bounds_min", F4), ("bounds_max", F4), ("metadata", U4)])
# GPUTextureDescriptor, 16 B
TEXTURE_DESCRIPTOR_DTYPE = np.dtype([("metadata", U4)])
# GPULightRecord, 32 B (GPUTypes.swift:54-60)
LIGHT_DTYPE = np.dtype([
    ("triangle_index", np.uint32), ("material_index", np.uint32),
    ("area", np.float32), ("selection_cdf", np.float32), ("normal", F4),
])
# GPUEnvironmentSample, 8 B (GPUTypes.swift:62-64)
ENVIRONMENT_SAMPLE_DTYPE = np.dtype([("cdf", np.float32), ("pdf_solid_angle", np.float32)])
# GPUVolumeDescriptor, 240 B (GPUTypes.swift:66-82)
VOLUME_DTYPE = np.dtype([
    ("world_bounds_min", F4), ("world_bounds_max", F4),
    ("local_bounds_min", F4), ("local_bounds_max", F4),
    ("dimensions", U4), ("metadata", U4), ("material_program", U4),
    ("world_to_local", (np.float32, (4, 4))), ("normal_transform", (np.float32, (4, 4))),
])
# GPUVolumeBrickSample, 16 B
BRICK_SAMPLE_DTYPE = np.dtype([
    ("distance", np.float32), ("material_a", np.uint32),
    ("material_b", np.uint32), ("material_blend", np.float32),
])
# GPUVolumeBrickDescriptor, 128 B
BRICK_DTYPE = np.dtype([
    ("world_bounds_min", F4), ("world_bounds_max", F4),
    ("local_bounds_min", F4), ("local_bounds_max", F4),
    ("sample_bounds_min", F4), ("sample_bounds_max", F4),
    ("grid_origin_and_volume", U4), ("dimensions_and_sample_offset", U4),
])
# GPUVolumeBrickGrid, 64 B
BRICK_GRID_DTYPE = np.dtype([
    ("dimensions_and_index_offset", U4), ("brick_size_and_volume", U4),
    ("macro_dimensions_and_index_offset", U4), ("macro_size_and_reserved", U4),
])

assert TRIANGLE_DTYPE.itemsize == 192
assert MATERIAL_DTYPE.itemsize == 272
assert NODE_DTYPE.itemsize == 48
assert LIGHT_DTYPE.itemsize == 32
assert ENVIRONMENT_SAMPLE_DTYPE.itemsize == 8
assert VOLUME_DTYPE.itemsize == 240
assert BRICK_DTYPE.itemsize == 128
assert BRICK_GRID_DTYPE.itemsize == 64


class Float4(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float), ("w", C.c_float)]


class Camera(C.Structure):
    """dk_camera / GPUCamera, 80 B."""
    _fields_ = [("origin", Float4), ("lower_left", Float4), ("horizontal", Float4),
                ("vertical", Float4), ("lens", Float4)]


_p = C.c_void_p


class Scene(C.Structure):
    """dk_scene: the AccelerationBuild arrays plus environment settings."""
    _fields_ = [
        ("triangles", _p), ("triangle_count", C.c_uint32),
        ("materials", _p), ("material_count", C.c_uint32),
        ("nodes", _p), ("node_count", C.c_uint32),
        ("primitive_indices", _p), ("primitive_index_count", C.c_uint32),
        ("texture_descriptors", _p), ("texture_descriptor_count", C.c_uint32),
        ("texture_pixels", _p), ("texture_pixel_count", C.c_uint64),
        ("lights", _p), ("light_count", C.c_uint32),
        ("environment_samples", _p), ("environment_sample_count", C.c_uint32),
        ("environment_texture_index_plus_one", C.c_uint32),
        ("environment_intensity", C.c_float),
        ("environment_rotation_y", C.c_float),
        ("environment_max_radiance", C.c_float),
        ("volumes", _p), ("volume_count", C.c_uint32),
        ("volume_bricks", _p), ("volume_brick_count", C.c_uint32),
        ("volume_brick_samples", _p), ("volume_brick_sample_count", C.c_uint64),
        ("volume_brick_grids", _p), ("volume_brick_grid_count", C.c_uint32),
        ("volume_brick_grid_indices", _p), ("volume_brick_grid_index_count", C.c_uint64),
    ]


class Settings(C.Structure):
    """dk_settings: RenderSettings plus the two cameras."""
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("max_bounces", C.c_uint32),
        ("quality", C.c_uint32), ("transparent_background", C.c_uint32),
        ("shows_environment_background", C.c_uint32), ("background_color", C.c_float * 3),
        ("sample_radiance_clamp_set", C.c_uint32), ("sample_radiance_clamp", C.c_float),
        ("frame_seed", C.c_uint32), ("denoiser_enabled", C.c_uint32),
        ("collects_traversal_stats", C.c_uint32),
        ("camera", Camera), ("previous_camera", Camera),
        ("max_samples_per_launch", C.c_uint32), ("triangle_test", C.c_uint32),
    ]


class Stats(C.Structure):
    """dk_stats."""
    _fields_ = [
        ("sdf_counters", C.c_uint64 * 13),
        ("paths_traced", C.c_uint64), ("rays_extended", C.c_uint64),
        ("shadow_rays", C.c_uint64), ("kernel_launches", C.c_uint64),
        ("last_render_ms", C.c_double), ("last_extend_ms", C.c_double),
        ("last_shade_ms", C.c_double), ("last_shadow_ms", C.c_double),
        ("last_other_ms", C.c_double), ("last_launches", C.c_uint64),
        ("device_bytes", C.c_uint64),
    ]


class OracleParams(C.Structure):
    """oracle_params of the CPU oracle (test infrastructure only)."""
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("max_bounces", C.c_uint32),
        ("transparent_background", C.c_uint32), ("shows_environment_background", C.c_uint32),
        ("background_color", C.c_float * 3), ("sample_radiance_clamp", C.c_float),
        ("frame_seed", C.c_uint32), ("denoiser_enabled", C.c_uint32),
        ("tile_x", C.c_uint32), ("tile_y", C.c_uint32), ("tile_w", C.c_uint32), ("tile_h", C.c_uint32),
        ("camera", Camera), ("previous_camera", Camera),
    ]


# dk_status (DenrimRendererError 1..5 + library codes)
STATUS_NAMES = {
    0: "DK_OK", 1: "DK_ERROR_NO_DEVICE", 2: "DK_ERROR_MISSING_KERNEL", 3: "DK_ERROR_INVALID_SCENE",
    4: "DK_ERROR_COMMAND_FAILED", 5: "DK_ERROR_EXPORT_FAILED", 6: "DK_ERROR_INVALID_ARGUMENT",
    7: "DK_ERROR_OUT_OF_MEMORY", 8: "DK_ERROR_DEVICE_TIMEOUT",
}

# Every symbol include/denrim_cuda.h declares (checked by tests/test_abi.py).
EXPORTED_SYMBOLS = (
    "dk_device_open", "dk_device_count", "dk_session_create", "dk_session_render",
    "dk_session_render_tile", "dk_session_update_camera", "dk_session_reset",
    "dk_session_read_output", "dk_session_copy_output", "dk_session_read_rgba8", "dk_session_write_png", "dk_encode_rgba8", "dk_write_png",
    "dk_session_sample_count", "dk_session_stats", "dk_session_reset_sdf_stats",
    "dk_session_destroy", "dk_last_error_message", "dk_build_bvh", "dk_build_lights",
    "dk_build_environment_samples", "dk_build_environment_samples_noalloc", "dk_build_sparse_sphere_volume",
    "dk_bake_sparse_sphere_volume",
    "dk_sparse_volume_view", "dk_sparse_volume_destroy", "dk_version", "dk_probe_bandwidth",
    "dk_server_create", "dk_server_add_scene", "dk_server_submit", "dk_server_step", "dk_server_start", "dk_server_stop",
    "dk_server_wait", "dk_server_job_status", "dk_server_read_output", "dk_server_copy_output", "dk_server_copy_outputs", "dk_server_release",
    "dk_server_get_stats", "dk_server_destroy", "dk_denoise_spatial", "dk_denoise_error_terms", "dk_average_planes", "dk_svgf_create", "dk_svgf_reset",
    "dk_svgf_denoise", "dk_svgf_read_state", "dk_svgf_destroy", "dk_svgf_pack_depth_normal", "dk_svgf_copy_output",
    "dk_unet_conv3x3", "dk_unet_conv3x3_avgpool2", "dk_unet_conv3x3_wgrad", "dk_unet_relu_backward", "dk_unet_bias_grad",
    "dk_unet_avgpool2",
    "dk_unet_avgpool2_backward", "dk_unet_upsample2", "dk_unet_upsample2_backward", "dk_unet_copy_channels",
    "dk_unet_pack_input", "dk_unet_l1_loss", "dk_unet_unpack_output", "dk_unet_l1_loss_residual",
    "dk_unet_unpack_output_residual", "dk_unet_adam", "dk_unet_weights_to_bf16",
    "dk_unet_set_conv_path", "dk_unet_error",
)


class SpatialDenoiseSettings(C.Structure):
    """dk_spatial_denoise_settings (DenoiseSettings defaults, Denoiser.swift:44-60)."""
    _fields_ = [("radius", C.c_uint32), ("normal_sigma", C.c_float), ("depth_sigma", C.c_float),
                ("albedo_sigma", C.c_float), ("color_sigma", C.c_float), ("iterations", C.c_uint32)]


class ServerConfig(C.Structure):
    """dk_server_config."""
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("wave_paths", C.c_uint32), ("max_jobs_per_wave", C.c_uint32),
                ("max_resident_jobs", C.c_uint32), ("samples_per_wave", C.c_uint32), ("policy", C.c_uint32),
                ("reserved", C.c_uint32)]


class JobDesc(C.Structure):
    """dk_job_desc."""
    _fields_ = [("settings", Settings), ("samples", C.c_uint32), ("material_count", C.c_uint32),
                ("materials", C.c_void_p), ("scene", C.c_uint32), ("reserved", C.c_uint32)]


class JobStatus(C.Structure):
    """dk_job_status."""
    _fields_ = [("job_id", C.c_uint64), ("state", C.c_uint32), ("samples_done", C.c_uint32),
                ("samples", C.c_uint32), ("waves", C.c_uint32), ("submit_ms", C.c_double),
                ("admit_ms", C.c_double), ("finish_ms", C.c_double)]


class ServerStats(C.Structure):
    """dk_server_stats."""
    _fields_ = [(k, C.c_uint64) for k in ("jobs_submitted", "jobs_done", "jobs_queued", "jobs_running", "waves",
                                          "paths_traced", "kernel_launches", "budget_used_bytes",
                                          "budget_peak_bytes", "device_bytes")] + \
               [("busy_ms", C.c_double), ("max_jobs_in_wave", C.c_double), ("mean_jobs_in_wave", C.c_double)]


JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_RELEASED = 0, 1, 2, 3


class SdfSphere(C.Structure):
    """dk_sdf_sphere."""
    _fields_ = [("center", C.c_float * 3), ("radius", C.c_float), ("material", C.c_uint32),
                ("smooth_union_radius", C.c_float)]


class SparseVolumeSettings(C.Structure):
    """dk_sparse_volume_settings."""
    _fields_ = [("resolution", C.c_uint32 * 3), ("bounds_min", C.c_float * 3), ("bounds_max", C.c_float * 3),
                ("brick_size", C.c_uint32 * 3), ("narrow_band", C.c_float), ("volume_material", C.c_uint32),
                ("object_id", C.c_uint32), ("primitive_id", C.c_uint32), ("fp16_distances", C.c_uint32)]

assert C.sizeof(Camera) == 80
