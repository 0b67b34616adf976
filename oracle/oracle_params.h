/* Test infrastructure: the per-render parameters shared by the CPU restatement
 * (pathtrace_oracle.cpp) and the host driver of the reference shader
 * (ref/ref_driver.cpp).  They are the values the reference packs into
 * GPURenderConstants (RenderSession.swift:908-947) plus the two cameras. */
#pragma once
#include <stdint.h>

#include "../include/denrim_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif
typedef struct oracle_params {
    uint32_t width, height, max_bounces;
    uint32_t transparent_background, shows_environment_background;
    float background_color[3];
    float sample_radiance_clamp; /* resolved (RenderSettings.resolvedSampleRadianceClamp) */
    uint32_t frame_seed;
    uint32_t denoiser_enabled;
    uint32_t tile_x, tile_y, tile_w, tile_h;
    dk_camera camera;
    dk_camera previous_camera;
} oracle_params;
#ifdef __cplusplus
}
#endif
